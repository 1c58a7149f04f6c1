/*
 * node_sort.c -- SortNode on the GPU (replaces src/sort.c; arrange()).
 *
 * sort_node_create returns a node with the reference's SortNode prefix
 * {base, child, n_keys, keys, phase, ...} and kind "SortNode", so the
 * optimizer re-points its key columns after pruning the child
 * (src/optimize.c:141-178) as it does on the reference's node; the keys are
 * read only when the node runs.
 *
 * next_batch pulls every batch of the child onto the device (columns laid
 * out densely, selection vectors applied), computes the stable order of
 * the rows by the keys (vgk_sort_rows: NA last ascending, first
 * descending, ties in input order -- the reference's merge sort,
 * src/sort.c:32-116), gathers every column in that order and returns one
 * malloc-owned batch, then NULL: the reference's in-memory result
 * (src/sort.c:488-529), an empty batch included.  Where the reference
 * spills runs beyond its 1 GiB budget and merges them in 65,536-row
 * batches, this node keeps everything in HBM and still returns one batch.
 * A string key sorts by the rank of its string among the column's
 * distinct strings (a device dictionary, ordered by memcmp with the
 * shorter string first, the reference's string compare); string columns
 * travel as device views into the child's batches, which stay resident
 * until the output is copied out.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "vg_host.h"

typedef struct {
    SortNode sn;                 /* reference prefix */
} VgSort;

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }
static size_t elem(int type) { return type == VEC_BOOL ? 1 : type == VEC_STRING ? 16 : 8; }

static VecBatch *sort_next_body(VecNode *self) {
    VgSort *S = (VgSort *)self;
    if (S->sn.phase == 3) return NULL;
    S->sn.phase = 3;
    VecNode *child = S->sn.child;
    const VecSchema *cs = &child->output_schema;
    const int nc = cs->n_cols;
    for (int k = 0; k < S->sn.n_keys; k++)
        if (S->sn.keys[k].col_index < 0 || S->sn.keys[k].col_index >= nc)
            vg_fail("sort: key column %d out of range", S->sn.keys[k].col_index);

    /* every batch of the child on the device */
    uint8_t *need = (uint8_t *)vg_xcalloc((size_t)(nc ? nc : 1), 1);
    memset(need, 1, (size_t)(nc ? nc : 1));
    int nb = 0, cap = 16;
    VgDBatch *bs = (VgDBatch *)vg_xcalloc((size_t)cap, sizeof(VgDBatch));
    int64_t total = 0;
    for (;;) {
        if (nb == cap) {
            cap *= 2;
            VgDBatch *nbs = (VgDBatch *)realloc(bs, (size_t)cap * sizeof(VgDBatch));
            if (!nbs) vg_fail("host allocation failed");
            bs = nbs;
        }
        if (!vg_pull(child, need, 0, &bs[nb])) break;
        total += bs[nb].d_sel ? bs[nb].sel_n : bs[nb].n_rows;
        nb++;
    }
    free(need);
    if (total > (int64_t)2147483647)
        vg_fail("sort: %lld rows; the GPU sort orders at most 2^31-1 rows", (long long)total);

    /* dense device columns of the logical rows */
    const size_t wbytes = (size_t)((total + 31) / 32) * 4 + 8;
    size_t bytes = 256;
    for (int c = 0; c < nc; c++) bytes += a256((size_t)total * elem(cs->col_types[c]) + 8) + a256(wbytes);
    char *blk = (char *)vg_dmalloc(bytes);
    VgCol *cols = (VgCol *)vg_xcalloc((size_t)(nc ? nc : 1), sizeof(VgCol));
    size_t off = 0;
    for (int c = 0; c < nc; c++) {
        char *dv = blk + off;
        off += a256((size_t)total * elem(cs->col_types[c]) + 8);
        uint32_t *dm = (uint32_t *)(blk + off);
        off += a256(wbytes);
        vg_dmemset(dm, 0, wbytes);
        int64_t at = 0;
        for (int b = 0; b < nb; b++) {
            const int64_t n = bs[b].d_sel ? bs[b].sel_n : bs[b].n_rows;
            if (n == 0) continue;
            if ((at & 31) == 0)
                vg_check_rc(vgk_gather(&bs[b].cols[c], bs[b].d_sel, n, 0, dv + (size_t)at * elem(cs->col_types[c]),
                                       dm + at / 32, vg_stream()), "sort gather");
            else
                vg_check_rc(vgk_gather_into(&bs[b].cols[c], bs[b].d_sel, n, dv, dm, at, vg_stream()), "sort gather");
            at += n;
        }
        cols[c].type = cs->col_types[c];
        cols[c].data = dv;
        cols[c].valid = dm;
        cols[c].voff = 0;
    }
    /* the order, then every column gathered in it */
    VecBatch *out = vg_batch_alloc(nc, total);
    for (int c = 0; c < nc; c++) out->col_names[c] = vg_xstrdup(cs->col_names[c]);
    if (total > 0) {
        const int nk = S->sn.n_keys;
        int *kc = (int *)vg_xcalloc((size_t)(nk ? nk : 1), sizeof(int));
        int *kd = (int *)vg_xcalloc((size_t)(nk ? nk : 1), sizeof(int));
        /* sort columns: the columns themselves, then one rank column per string key */
        VgCol *sc = (VgCol *)vg_xcalloc((size_t)(nc + nk + 1), sizeof(VgCol));
        for (int c = 0; c < nc; c++) sc[c] = cols[c];
        int n_sc = nc;
        char *ranks = NULL;
        for (int k = 0; k < nk; k++) {
            kc[k] = S->sn.keys[k].col_index;
            kd[k] = S->sn.keys[k].descending != 0;
            if (cols[kc[k]].type != VEC_STRING) continue;
            if (!ranks) ranks = (char *)vg_dmalloc(a256((size_t)total * 8) * (size_t)(nk + 1) + 256);
            int64_t *codes = (int64_t *)(ranks + a256((size_t)total * 8) * (size_t)nk);
            int64_t *rk = (int64_t *)(ranks + a256((size_t)total * 8) * (size_t)k);
            VgDict *D = vg_dict_new();
            vg_dict_encode(D, &cols[kc[k]], NULL, total, 1, codes);
            int32_t *dperm = NULL;
            int64_t *drank = NULL;
            vg_dict_order(D, &dperm, &drank);
            vg_check_rc(vgk_map_codes(drank, codes, cols[kc[k]].valid, 0, total, rk, vg_stream()), "sort");
            vg_dfree(dperm);
            vg_dfree(drank);
            vg_dict_free(D);
            sc[n_sc].type = VEC_INT64;
            sc[n_sc].data = rk;
            sc[n_sc].valid = cols[kc[k]].valid;
            kc[k] = n_sc++;
        }
        const size_t sb = vgk_sort_rows_scratch(total);
        char *work = (char *)vg_dmalloc(sb + (size_t)total * 4 + 256);
        int32_t *perm = (int32_t *)(work + sb);
        vg_check_rc(vgk_sort_rows(sc, kc, kd, nk, perm, total, work, sb, vg_stream()), "sort");
        vg_dfree(ranks);
        free(sc);
        free(kc);
        free(kd);
        const size_t ob = a256((size_t)total * 16 + 8) + a256(wbytes);
        char *ob_blk = (char *)vg_dmalloc(ob);
        for (int c = 0; c < nc; c++) {
            uint32_t *om = (uint32_t *)(ob_blk + a256((size_t)total * 16 + 8));
            vg_check_rc(vgk_gather(&cols[c], perm, total, 0, ob_blk, om, vg_stream()), "sort gather");
            if (cs->col_types[c] == VEC_STRING) {
                VgCol v;
                memset(&v, 0, sizeof(v));
                v.type = VEC_STRING;
                v.data = ob_blk;
                v.valid = om;
                out->columns[c] = vg_download_strings(&v, NULL, total);
            } else {
                out->columns[c] = vg_download_column(cs->col_types[c], ob_blk, om, total);
            }
        }
        vg_sync();
        vg_dfree(ob_blk);
        vg_dfree(work);
    } else {
        for (int c = 0; c < nc; c++) {
            VecArray a;
            memset(&a, 0, sizeof(a));
            a.type = (VecType)cs->col_types[c];
            a.owns_data = 1;
            a.validity = (uint8_t *)vg_xcalloc(1, 1);
            if (a.type == VEC_STRING) {
                a.buf.str.offsets = (int64_t *)vg_xcalloc(1, 8);
                a.buf.str.data = (char *)vg_xcalloc(1, 1);
            } else {
                a.buf.i64 = (int64_t *)vg_xcalloc(1, 8);
            }
            out->columns[c] = a;
        }
    }
    for (int b = 0; b < nb; b++) vg_dbatch_release(&bs[b]);   /* string views point into them */
    free(bs);
    vg_dfree(blk);
    free(cols);
    return out;
}

/* one node API call: its temporary device memory is released if it fails */
static VecBatch *sort_next(VecNode *self) {
    vg_scope_enter();
    VecBatch *b = sort_next_body(self);
    vg_scope_leave();
    return b;
}

static void sort_free(VecNode *self) {
    VgSort *S = (VgSort *)self;
    S->sn.child->free_node(S->sn.child);
    free(S->sn.keys);
    free(S->sn.temp_dir);
    vg_schema_free(&S->sn.base.output_schema);
    free(S);
}

SortNode *sort_node_create(VecNode *child, int n_keys, SortKey *keys, const char *temp_dir) {
    VgSort *S = (VgSort *)vg_xcalloc(1, sizeof(VgSort));
    S->sn.child = child;
    S->sn.n_keys = n_keys;
    S->sn.keys = keys;
    S->sn.phase = 0;
    S->sn.mem_budget = 1024LL * 1024 * 1024;
    S->sn.temp_dir = temp_dir ? vg_xstrdup(temp_dir) : NULL;
    S->sn.base.output_schema = vg_schema_copy(&child->output_schema);
    S->sn.base.next_batch = sort_next;
    S->sn.base.free_node = sort_free;
    S->sn.base.kind = "SortNode";
    return &S->sn;
}
