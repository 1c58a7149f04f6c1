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
 * (src/sort.c:488-529), an empty batch included.  A string key sorts by
 * the rank of its string among the column's distinct strings (a device
 * dictionary, ordered by memcmp with the shorter string first, the
 * reference's string compare); string columns travel as device views into
 * the child's batches, which stay resident until the output is copied out.
 *
 * Beyond device memory (the reference spills sorted runs past its 1 GiB
 * budget and merges them from disk, src/sort.c:349-470, 566-636): the
 * input is cut into runs that each fit a device budget; each run is sorted
 * on the device and kept in host memory.  The runs are then merged by key
 * range: splitters sampled from the runs cut every run into slices (host
 * binary searches, a few per splitter); each key range's slices go back to
 * the device in run order, are sorted there (stably, so equal keys keep
 * run order, then row order: the input order) and are copied into their
 * place in the output.  A range of one repeated key larger than the budget
 * needs no sort and is copied in run order.  The output is still one
 * batch.  The budget is a share of the free device memory, or
 * VGPU_SORT_RUN_ROWS rows.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "vg_host.h"

typedef struct {
    SortNode sn;                 /* reference prefix */
} VgSort;

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }
static size_t elem(int type) { return type == VEC_BOOL ? 1 : type == VEC_STRING ? 16 : 8; }

/* runs sorted into host memory and key ranges merged, since load */
static long g_sort_runs, g_sort_ranges;
long vgpu_sort_spill_stats(long *ranges) {
    if (ranges) *ranges = g_sort_ranges;
    return g_sort_runs;
}

/* ------------------------------------------------------------------ */
/* device columns, order, output                                       */
/* ------------------------------------------------------------------ */

/* Dense device columns of the logical rows of bs[0..nb) (values, then
 * validity words), in one new block *blk. */
static void dense_from_batches(VgDBatch *bs, int nb, int64_t total, const VecSchema *cs, VgCol *cols, char **blk) {
    const int nc = cs->n_cols;
    const size_t wbytes = (size_t)((total + 31) / 32) * 4 + 8;
    size_t bytes = 256;
    for (int c = 0; c < nc; c++) bytes += a256((size_t)total * elem(cs->col_types[c]) + 8) + a256(wbytes);
    char *b = (char *)vg_dmalloc(bytes);
    size_t off = 0;
    for (int c = 0; c < nc; c++) {
        char *dv = b + off;
        off += a256((size_t)total * elem(cs->col_types[c]) + 8);
        uint32_t *dm = (uint32_t *)(b + off);
        off += a256(wbytes);
        vg_dmemset(dm, 0, wbytes);
        int64_t at = 0;
        for (int i = 0; i < nb; i++) {
            const int64_t n = bs[i].d_sel ? bs[i].sel_n : bs[i].n_rows;
            if (n == 0) continue;
            if ((at & 31) == 0)
                vg_check_rc(vgk_gather(&bs[i].cols[c], bs[i].d_sel, n, 0, dv + (size_t)at * elem(cs->col_types[c]),
                                       dm + at / 32, vg_stream()), "sort gather");
            else
                vg_check_rc(vgk_gather_into(&bs[i].cols[c], bs[i].d_sel, n, dv, dm, at, vg_stream()), "sort gather");
            at += n;
        }
        cols[c].type = cs->col_types[c];
        cols[c].data = dv;
        cols[c].valid = dm;
        cols[c].voff = 0;
    }
    *blk = b;
}

/* The stable order of n rows of cols by the node's keys: a device
 * permutation inside *work (freed by the caller). */
static int32_t *order_rows(VgSort *S, const VgCol *cols, int nc, int64_t n, char **work) {
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
        if (!ranks) ranks = (char *)vg_dmalloc(a256((size_t)n * 8) * (size_t)(nk + 1) + 256);
        int64_t *codes = (int64_t *)(ranks + a256((size_t)n * 8) * (size_t)nk);
        int64_t *rk = (int64_t *)(ranks + a256((size_t)n * 8) * (size_t)k);
        VgDict *D = vg_dict_new();
        vg_dict_encode(D, &cols[kc[k]], NULL, n, 1, codes, -1);
        int32_t *dperm = NULL;
        int64_t *drank = NULL;
        vg_dict_order(D, &dperm, &drank);
        vg_check_rc(vgk_map_codes(drank, codes, cols[kc[k]].valid, cols[kc[k]].voff, n, rk, vg_stream()), "sort");
        vg_dfree(dperm);
        vg_dfree(drank);
        vg_dict_free(D);
        sc[n_sc].type = VEC_INT64;
        sc[n_sc].data = rk;
        sc[n_sc].valid = cols[kc[k]].valid;
        sc[n_sc].voff = cols[kc[k]].voff;
        kc[k] = n_sc++;
    }
    const size_t sb = vgk_sort_rows_scratch(n);
    char *w = (char *)vg_dmalloc(sb + (size_t)n * 4 + 256);
    int32_t *perm = (int32_t *)(w + sb);
    vg_check_rc(vgk_sort_rows(sc, kc, kd, nk, perm, n, w, sb, vg_stream()), "sort");
    vg_dfree(ranks);
    free(sc);
    free(kc);
    free(kd);
    *work = w;
    return perm;
}

/* dst bits [at, at + n) = src bits [0, n) (reference bitmap order) */
static void put_bits(uint8_t *dst, int64_t at, const uint8_t *src, int64_t n) {
    if ((at & 7) == 0) {
        memcpy(dst + at / 8, src, (size_t)vg_vbytes(n));
        return;
    }
    for (int64_t i = 0; i < n; i++) {
        const int64_t d = at + i;
        if ((src[i >> 3] >> (i & 7)) & 1) dst[d >> 3] |= (uint8_t)(1u << (d & 7));
        else dst[d >> 3] &= (uint8_t)~(1u << (d & 7));
    }
}

/* An output batch of n rows (validity clear; string columns with room for
 * cap[c] bytes of characters, cap updated as emit_rows grows them). */
static VecBatch *out_alloc(const VecSchema *cs, int64_t n, int64_t *cap) {
    VecBatch *out = vg_batch_alloc(cs->n_cols, n);
    for (int c = 0; c < cs->n_cols; c++) {
        VecArray *a = &out->columns[c];
        a->type = (VecType)cs->col_types[c];
        a->length = n;
        a->owns_data = 1;
        a->validity = (uint8_t *)vg_xcalloc((size_t)vg_vbytes(n) + 1, 1);
        if (a->type == VEC_STRING) {
            a->buf.str.offsets = (int64_t *)vg_xcalloc((size_t)n + 1, 8);
            a->buf.str.data = (char *)vg_xmalloc((size_t)cap[c] + 1);
            a->buf.str.data_len = 0;
        } else {
            a->buf.i64 = (int64_t *)vg_xcalloc((size_t)n * (a->type == VEC_BOOL ? 1 : 8) + 8, 1);
        }
        out->col_names[c] = vg_xstrdup(cs->col_names[c]);
    }
    return out;
}

/* rows perm[0..n) of cols (perm NULL: rows 0..n-1) into rows [at, at + n)
 * of out; a string column's characters are appended at its data_len */
static void emit_rows(const VgCol *cols, int nc, const int32_t *perm, int64_t n, VecBatch *out, int64_t at,
                      int64_t *cap) {
    if (n <= 0) return;
    const size_t wb = (size_t)((n + 31) / 32) * 4 + 8;
    char *ob = (char *)vg_dmalloc(a256((size_t)n * 16 + 8) + a256(wb));
    uint32_t *om = (uint32_t *)(ob + a256((size_t)n * 16 + 8));
    uint8_t *hv = (uint8_t *)vg_xmalloc(wb);
    for (int c = 0; c < nc; c++) {
        VecArray *a = &out->columns[c];
        vg_check_rc(vgk_gather(&cols[c], perm, n, 0, ob, om, vg_stream()), "sort gather");
        if (cols[c].type == VEC_STRING) {
            VgCol v;
            memset(&v, 0, sizeof(v));
            v.type = VEC_STRING;
            v.data = ob;
            v.valid = om;
            VecArray p = vg_download_strings(&v, NULL, n);
            const int64_t base = a->buf.str.data_len;
            if (base + p.buf.str.data_len > cap[c]) {
                int64_t nc2 = cap[c] ? 2 * cap[c] : 4096;
                while (nc2 < base + p.buf.str.data_len) nc2 *= 2;
                char *d = (char *)realloc(a->buf.str.data, (size_t)nc2 + 1);
                if (!d) vg_fail("host allocation failed");
                a->buf.str.data = d;
                cap[c] = nc2;
            }
            memcpy(a->buf.str.data + base, p.buf.str.data, (size_t)p.buf.str.data_len);
            for (int64_t i = 0; i <= n; i++) a->buf.str.offsets[at + i] = base + p.buf.str.offsets[i];
            a->buf.str.data_len = base + p.buf.str.data_len;
            put_bits(a->validity, at, p.validity, n);
            free(p.validity);
            free(p.buf.str.offsets);
            free(p.buf.str.data);
        } else {
            const size_t es = cols[c].type == VEC_BOOL ? 1 : 8;
            vg_d2h((char *)(cols[c].type == VEC_BOOL ? (void *)a->buf.bln : (void *)a->buf.i64) + (size_t)at * es, ob,
                   (size_t)n * es);
            vg_d2h(hv, om, (size_t)vg_vbytes(n));
            vg_sync();
            put_bits(a->validity, at, hv, n);
        }
    }
    free(hv);
    vg_dfree(ob);
}

/* ------------------------------------------------------------------ */
/* beyond device memory: sorted runs in host memory, merged by range   */
/* ------------------------------------------------------------------ */

/* rows per run: VGPU_SORT_RUN_ROWS, else about a third of the free device
 * memory over the bytes a row takes on the device while it is sorted */
static int64_t run_budget(const VecSchema *cs, int n_keys) {
    const int64_t most = 2147483647;     /* a device sort orders at most 2^31-1 rows */
    const char *e = getenv("VGPU_SORT_RUN_ROWS");
    if (e && atoll(e) > 0) return atoll(e) < most ? atoll(e) : most;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess || fr == 0) return most;
    size_t row = 64 + 40 * (size_t)n_keys;
    for (int c = 0; c < cs->n_cols; c++)
        row += 3 * elem(cs->col_types[c]) + 1 + (cs->col_types[c] == VEC_STRING ? 64 : 0);
    const int64_t r = (int64_t)(fr / 3 / row);
    return r < 1024 ? 1024 : r > most ? most : r;
}

/* the order word of a valid fixed-width value, as the device sort forms it */
static uint64_t host_word(const VecArray *a, int64_t r) {
    if (a->type == VEC_BOOL) return a->buf.bln[r];
    uint64_t b;
    memcpy(&b, &a->buf.i64[r], 8);
    if (a->type == VEC_DOUBLE) {
        if (b == 0x8000000000000000ull) b = 0;
        return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
    }
    return b ^ 0x8000000000000000ull;
}

static int host_valid(const VecArray *a, int64_t r) { return !a->validity || ((a->validity[r >> 3] >> (r & 7)) & 1); }

/* key order of row ra of batch A against row rb of batch B: the device
 * sort's order (NA last ascending, first descending) */
static int key_cmp(const VgSort *S, const VecBatch *A, int64_t ra, const VecBatch *B, int64_t rb) {
    for (int k = 0; k < S->sn.n_keys; k++) {
        const int c = S->sn.keys[k].col_index, desc = S->sn.keys[k].descending != 0;
        const VecArray *x = &A->columns[c], *y = &B->columns[c];
        const int vx = host_valid(x, ra), vy = host_valid(y, rb);
        if (!vx || !vy) {
            if (vx == vy) continue;
            return !vx ? (desc ? -1 : 1) : (desc ? 1 : -1);
        }
        int r;
        if (x->type == VEC_STRING) {
            const int64_t sa = x->buf.str.offsets[ra], la = x->buf.str.offsets[ra + 1] - sa;
            const int64_t sb = y->buf.str.offsets[rb], lb = y->buf.str.offsets[rb + 1] - sb;
            r = memcmp(x->buf.str.data + sa, y->buf.str.data + sb, (size_t)(la < lb ? la : lb));
            r = r < 0 ? -1 : r > 0 ? 1 : (la > lb) - (la < lb);
        } else {
            const uint64_t wx = host_word(x, ra), wy = host_word(y, rb);
            r = (wx > wy) - (wx < wy);
        }
        if (r) return desc ? -r : r;
    }
    return 0;
}

typedef struct { int run; int64_t row; } RowRef;

/* the first row of R in [lo, hi) whose key is not below row rb of B */
static int64_t lower_bound(const VgSort *S, const VecBatch *R, int64_t lo, int64_t hi, const VecBatch *B, int64_t rb) {
    while (lo < hi) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (key_cmp(S, R, mid, B, rb) < 0) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

static const VgSort *g_cmp_sort;
static VecBatch **g_cmp_runs;
static int ref_cmp(const void *a, const void *b) {
    const RowRef *x = (const RowRef *)a, *y = (const RowRef *)b;
    const int r = key_cmp(g_cmp_sort, g_cmp_runs[x->run], x->row, g_cmp_runs[y->run], y->row);
    if (r) return r;
    return x->run != y->run ? (x->run < y->run ? -1 : 1) : (x->row > y->row) - (x->row < y->row);
}

typedef struct {
    VgSort *S;
    const VecSchema *cs;
    VecBatch **runs;
    int nr;
    int64_t budget;
    VecBatch *out;
    int64_t out_at;
    int64_t *cap;
} Merge;

/* rows [lo, lo + m) of run r to the output as they are (device copies) */
static void copy_slice(Merge *M, int r, int64_t lo, int64_t m) {
    const int nc = M->cs->n_cols;
    VgCol *cols = (VgCol *)vg_xcalloc((size_t)(nc ? nc : 1), sizeof(VgCol));
    void **blks = (void **)vg_xcalloc((size_t)(nc ? nc : 1), sizeof(void *));
    for (int c = 0; c < nc; c++) cols[c] = vg_upload_slice(&M->runs[r]->columns[c], lo, m, &blks[c]);
    emit_rows(cols, nc, NULL, m, M->out, M->out_at, M->cap);
    M->out_at += m;
    for (int c = 0; c < nc; c++) vg_dfree(blks[c]);
    free(cols);
    free(blks);
}

/* One key range: rows [lo[r], hi[r]) of every run r, in order, to the
 * output.  Sorted on the device when it fits the budget; otherwise cut by
 * splitters sampled from it, or -- one repeated key -- copied in run
 * order. */
static void merge_range(Merge *M, const int64_t *lo, const int64_t *hi) {
    const int nr = M->nr, nc = M->cs->n_cols;
    int64_t n = 0;
    for (int r = 0; r < nr; r++) n += hi[r] - lo[r];
    if (n == 0) return;
    if (n > M->budget) {
        /* the least and the greatest key of the range */
        int rmin = -1, rmax = -1;
        for (int r = 0; r < nr; r++) {
            if (hi[r] <= lo[r]) continue;
            if (rmin < 0 || key_cmp(M->S, M->runs[r], lo[r], M->runs[rmin], lo[rmin]) < 0) rmin = r;
            if (rmax < 0 || key_cmp(M->S, M->runs[r], hi[r] - 1, M->runs[rmax], hi[rmax] - 1) > 0) rmax = r;
        }
        if (key_cmp(M->S, M->runs[rmin], lo[rmin], M->runs[rmax], hi[rmax] - 1) != 0) {
            /* splitters: 64 samples per part, parts of about half the budget */
            const int64_t parts = (2 * n + M->budget - 1) / M->budget + 1;
            const int64_t want = parts * 64;
            RowRef *smp = (RowRef *)vg_xcalloc((size_t)(want + nr), sizeof(RowRef));
            int64_t ns = 0;
            for (int r = 0; r < nr; r++) {
                const int64_t len = hi[r] - lo[r];
                if (len <= 0) continue;
                const int64_t k = (len * want + n - 1) / n;
                for (int64_t i = 0; i < k && ns < want + nr; i++) {
                    smp[ns].run = r;
                    smp[ns].row = lo[r] + (i * len) / k;
                    ns++;
                }
            }
            g_cmp_sort = M->S;
            g_cmp_runs = M->runs;
            qsort(smp, (size_t)ns, sizeof(RowRef), ref_cmp);
            int64_t *b = (int64_t *)vg_xcalloc((size_t)(parts + 1) * (size_t)nr, sizeof(int64_t));
            for (int r = 0; r < nr; r++) {
                b[r] = lo[r];
                b[(size_t)parts * nr + r] = hi[r];
            }
            for (int64_t p = 1; p < parts; p++) {
                const RowRef *sp = &smp[p * ns / parts];
                for (int r = 0; r < nr; r++)
                    b[(size_t)p * nr + r] =
                        lower_bound(M->S, M->runs[r], b[(size_t)(p - 1) * nr + r], hi[r], M->runs[sp->run], sp->row);
            }
            free(smp);
            /* recurse only when every part is smaller than the range */
            int progress = 1;
            for (int64_t p = 0; p < parts; p++) {
                int64_t m = 0;
                for (int r = 0; r < nr; r++) m += b[(size_t)(p + 1) * nr + r] - b[(size_t)p * nr + r];
                if (m == n) progress = 0;
            }
            if (!progress) {
                /* the samples missed every key but one: cut below the
                 * greatest key instead (both sides then hold rows) */
                for (int r = 0; r < nr; r++) {
                    b[r] = lo[r];
                    b[(size_t)nr + r] = lower_bound(M->S, M->runs[r], lo[r], hi[r], M->runs[rmax], hi[rmax] - 1);
                    b[(size_t)2 * nr + r] = hi[r];
                }
                merge_range(M, b, b + nr);
                merge_range(M, b + nr, b + 2 * (size_t)nr);
                free(b);
                return;
            }
            for (int64_t p = 0; p < parts; p++) merge_range(M, b + (size_t)p * nr, b + (size_t)(p + 1) * nr);
            free(b);
            return;
        }
        /* one repeated key: run order, then each run's own order */
        for (int r = 0; r < nr; r++)
            for (int64_t s = lo[r]; s < hi[r]; s += M->budget)
                copy_slice(M, r, s, hi[r] - s < M->budget ? hi[r] - s : M->budget);
        g_sort_ranges++;
        return;
    }
    /* the range's slices on the device in run order, dense */
    const size_t wbytes = (size_t)((n + 31) / 32) * 4 + 8;
    size_t bytes = 256;
    for (int c = 0; c < nc; c++) bytes += a256((size_t)n * elem(M->cs->col_types[c]) + 8) + a256(wbytes);
    char *blk = (char *)vg_dmalloc(bytes);
    VgCol *cols = (VgCol *)vg_xcalloc((size_t)(nc ? nc : 1), sizeof(VgCol));
    void **sblk = (void **)vg_xcalloc((size_t)(nc ? nc : 1) * (size_t)nr, sizeof(void *));
    size_t off = 0;
    for (int c = 0; c < nc; c++) {
        char *dv = blk + off;
        off += a256((size_t)n * elem(M->cs->col_types[c]) + 8);
        uint32_t *dm = (uint32_t *)(blk + off);
        off += a256(wbytes);
        vg_dmemset(dm, 0, wbytes);
        int64_t at = 0;
        for (int r = 0; r < nr; r++) {
            const int64_t m = hi[r] - lo[r];
            if (m <= 0) continue;
            const VgCol sc = vg_upload_slice(&M->runs[r]->columns[c], lo[r], m, &sblk[(size_t)c * nr + r]);
            vg_check_rc(vgk_gather_into(&sc, NULL, m, dv, dm, at, vg_stream()), "sort merge");
            at += m;
        }
        cols[c].type = M->cs->col_types[c];
        cols[c].data = dv;
        cols[c].valid = dm;
    }
    char *work = NULL;
    const int32_t *perm = order_rows(M->S, cols, nc, n, &work);
    emit_rows(cols, nc, perm, n, M->out, M->out_at, M->cap);
    M->out_at += n;
    vg_dfree(work);
    for (size_t i = 0; i < (size_t)(nc ? nc : 1) * (size_t)nr; i++) vg_dfree(sblk[i]);
    free(sblk);
    free(cols);
    vg_dfree(blk);
    g_sort_ranges++;
}

/* ------------------------------------------------------------------ */
/* the node                                                            */
/* ------------------------------------------------------------------ */

/* bs[0..nb) (total logical rows) sorted into a new host batch */
static VecBatch *sort_batches(VgSort *S, const VecSchema *cs, VgDBatch *bs, int nb, int64_t total) {
    const int nc = cs->n_cols;
    if (total > (int64_t)2147483647)
        vg_fail("sort: %lld rows in device memory at once; the GPU sort orders at most 2^31-1", (long long)total);
    VgCol *cols = (VgCol *)vg_xcalloc((size_t)(nc ? nc : 1), sizeof(VgCol));
    char *blk = NULL;
    dense_from_batches(bs, nb, total, cs, cols, &blk);
    int64_t *cap = (int64_t *)vg_xcalloc((size_t)(nc ? nc : 1), sizeof(int64_t));
    VecBatch *out = out_alloc(cs, total, cap);
    if (total > 0) {
        char *work = NULL;
        const int32_t *perm = order_rows(S, cols, nc, total, &work);
        emit_rows(cols, nc, perm, total, out, 0, cap);
        vg_dfree(work);
    }
    free(cap);
    vg_dfree(blk);
    free(cols);
    return out;
}

static VecBatch **push_run(VecBatch **runs, int *nr, int *rcap, VecBatch *b) {
    if (*nr == *rcap) {
        *rcap *= 2;
        VecBatch **n2 = (VecBatch **)realloc(runs, (size_t)*rcap * sizeof(VecBatch *));
        if (!n2) vg_fail("host allocation failed");
        runs = n2;
    }
    runs[(*nr)++] = b;
    return runs;
}

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
    const int64_t budget = run_budget(cs, S->sn.n_keys);

    /* every batch of the child on the device; the batches so far sorted
     * into a host run whenever the next one would pass the budget */
    uint8_t *need = (uint8_t *)vg_xcalloc((size_t)(nc ? nc : 1), 1);
    memset(need, 1, (size_t)(nc ? nc : 1));
    int nb = 0, cap = 16, nr = 0, rcap = 8;
    VgDBatch *bs = (VgDBatch *)vg_xcalloc((size_t)cap, sizeof(VgDBatch));
    VecBatch **runs = (VecBatch **)vg_xcalloc((size_t)rcap, sizeof(VecBatch *));
    int64_t in_run = 0, total = 0;
    for (;;) {
        if (nb == cap) {
            cap *= 2;
            VgDBatch *nbs = (VgDBatch *)realloc(bs, (size_t)cap * sizeof(VgDBatch));
            if (!nbs) vg_fail("host allocation failed");
            bs = nbs;
        }
        if (!vg_pull(child, need, 0, &bs[nb])) break;
        const int64_t n = bs[nb].d_sel ? bs[nb].sel_n : bs[nb].n_rows;
        if (in_run > 0 && in_run + n > budget) {
            const VgDBatch next = bs[nb];
            runs = push_run(runs, &nr, &rcap, sort_batches(S, cs, bs, nb, in_run));
            for (int i = 0; i < nb; i++) vg_dbatch_release(&bs[i]);
            bs[0] = next;
            nb = 0;
            in_run = 0;
        }
        in_run += n;
        total += n;
        nb++;
    }
    free(need);
    if (nr == 0) {                       /* everything fit: one device sort */
        VecBatch *out = sort_batches(S, cs, bs, nb, in_run);
        for (int i = 0; i < nb; i++) vg_dbatch_release(&bs[i]);
        free(bs);
        free(runs);
        return out;
    }
    if (nb > 0) runs = push_run(runs, &nr, &rcap, sort_batches(S, cs, bs, nb, in_run));
    for (int i = 0; i < nb; i++) vg_dbatch_release(&bs[i]);
    free(bs);
    g_sort_runs += nr;

    /* merge by key range into one output batch */
    Merge M;
    memset(&M, 0, sizeof(M));
    M.S = S;
    M.cs = cs;
    M.runs = runs;
    M.nr = nr;
    M.budget = budget;
    M.cap = (int64_t *)vg_xcalloc((size_t)(nc ? nc : 1), sizeof(int64_t));
    for (int c = 0; c < nc; c++)
        if (cs->col_types[c] == VEC_STRING)
            for (int r = 0; r < nr; r++) M.cap[c] += runs[r]->columns[c].buf.str.data_len;
    M.out = out_alloc(cs, total, M.cap);
    int64_t *lo = (int64_t *)vg_xcalloc((size_t)nr, sizeof(int64_t));
    int64_t *hi = (int64_t *)vg_xcalloc((size_t)nr, sizeof(int64_t));
    for (int r = 0; r < nr; r++) hi[r] = runs[r]->n_rows;
    merge_range(&M, lo, hi);
    free(lo);
    free(hi);
    free(M.cap);
    for (int r = 0; r < nr; r++) vg_batch_free(runs[r]);
    free(runs);
    if (M.out_at != total) vg_fail("sort: merged %lld of %lld rows", (long long)M.out_at, (long long)total);
    return M.out;
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
