/*
 * strdict.c -- string dictionaries on the device (host side).
 *
 * A dictionary gives every distinct string of a column a dense int64 code
 * (k_strings.cu), so that a string group key runs through the group-agg's
 * integer key path: each batch's string column is replaced by its codes
 * before the aggregation kernel reads it, and the output maps the groups'
 * codes back to strings.  Where the reference keeps the bytes of every
 * group key in its key arena and compares them on each probe
 * (src/group_agg.c:18-149, src/hash.c:35-43, 58-66), the bytes of each
 * distinct string are hashed, compared and copied once.
 *
 * Before each encode the dictionary makes room for every row of the batch
 * (codes, arena bytes, a slot table at most half full), so the device
 * never runs out of space mid-launch.  Its error word (a bounded wait that
 * ran out) is read with the next batch's counters and at the end.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "vg_host.h"

struct VgDict {
    VgStrDict d;
    unsigned long long *d_ctr;       /* VG_DICT_CTRS counters, then the error word */
    unsigned long long h_ctr[VG_DICT_CTRS + 1];
    int kept;                        /* outlives the node call that made it */
    /* upper bounds of the device's code and arena counters since they were
     * last read: launches whose rows fit under the capacity by these need
     * no read-back first */
    int64_t ub_codes, ub_used;
};

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

static void *dalloc(VgDict *D, size_t bytes) { return D->kept ? vg_dmalloc_kept(bytes) : vg_dmalloc(bytes); }

static VgDict *dict_new(int kept) {
    VgDict *D = (VgDict *)vg_xcalloc(1, sizeof(VgDict));
    D->kept = kept;
    D->d_ctr = (unsigned long long *)dalloc(D, (VG_DICT_CTRS + 1) * 8);
    vg_dmemset(D->d_ctr, 0, (VG_DICT_CTRS + 1) * 8);
    D->d.ctr = D->d_ctr;
    return D;
}

VgDict *vg_dict_new(void) { return dict_new(0); }

/* for a node that keeps the dictionary across its calls (a join's keys) */
VgDict *vg_dict_new_kept(void) { return dict_new(1); }

void vg_dict_free(VgDict *D) {
    if (!D) return;
    vg_dfree(D->d.slot);
    vg_dfree(D->d.c_hash);
    vg_dfree(D->d.c_off);
    vg_dfree(D->d.c_len);
    vg_dfree(D->d.arena);
    vg_dfree(D->d_ctr);
    free(D);
}

static uint32_t *err_word(VgDict *D) { return (uint32_t *)(D->d_ctr + VG_DICT_CTRS); }

/* counters and error word to the host (one wait) */
static void dict_read(VgDict *D) {
    vg_d2h(D->h_ctr, D->d_ctr, (VG_DICT_CTRS + 1) * 8);
    vg_sync();
    const uint32_t err = (uint32_t)D->h_ctr[VG_DICT_CTRS];
    if (err & VG_ERR_WAIT) vg_fail("string dictionary: a bounded device wait ran out");
    if (err) vg_fail("string dictionary: table full (error %u)", err);
}

static void *grow(VgDict *D, void *old, size_t used, size_t bytes) {
    void *p = dalloc(D, bytes);
    if (old && used) {
        const cudaError_t e = cudaMemcpyAsync(p, old, used, cudaMemcpyDeviceToDevice, (cudaStream_t)vg_stream());
        if (e != cudaSuccess) vg_fail("string dictionary: growing copy failed: %s", cudaGetErrorString(e));
    }
    vg_dfree(old);
    return p;
}

/* room for `rows` more codes and `bytes` more characters */
static void dict_reserve(VgDict *D, int64_t rows, int64_t bytes) {
    const int64_t n = (int64_t)D->h_ctr[VG_DICT_CODES], used = (int64_t)D->h_ctr[VG_DICT_USED];
    const int64_t need = n + rows;
    if (need > (int64_t)0x7FFFFFFF) vg_fail("string dictionary: more than 2^31-1 distinct strings");
    if (need > D->d.codes_cap) {
        int64_t cap = D->d.codes_cap ? 2 * D->d.codes_cap : 1024;
        while (cap < need) cap *= 2;
        D->d.c_hash = (uint64_t *)grow(D, D->d.c_hash, (size_t)n * 8, a256((size_t)cap * 8));
        D->d.c_off = (int64_t *)grow(D, D->d.c_off, (size_t)n * 8, a256((size_t)cap * 8));
        D->d.c_len = (uint32_t *)grow(D, D->d.c_len, (size_t)n * 4, a256((size_t)cap * 4));
        D->d.codes_cap = cap;
    }
    if (used + bytes > D->d.arena_cap) {
        int64_t cap = D->d.arena_cap ? 2 * D->d.arena_cap : (int64_t)1 << 16;
        while (cap < used + bytes) cap *= 2;
        D->d.arena = (char *)grow(D, D->d.arena, (size_t)used, a256((size_t)cap));
        D->d.arena_cap = cap;
    }
    if (D->d.cap == 0 || 2 * need > D->d.cap) {
        int64_t cap = D->d.cap ? 2 * D->d.cap : 2048;
        while (cap < 2 * need) cap *= 2;
        vg_dfree(D->d.slot);
        D->d.slot = (uint32_t *)dalloc(D, a256((size_t)cap * 4));
        D->d.cap = cap;
        vg_check_rc(vgk_dict_rehash(&D->d, n, err_word(D), vg_stream()), "string dictionary");
    }
}

void vg_dict_encode(VgDict *D, const VgCol *c, const int32_t *d_sel, int64_t n_logical, int insert,
                    int64_t *d_codes, int64_t chars_ub) {
    if (n_logical <= 0) return;
    if (insert && chars_ub >= 0) {
        /* every row may be new: room for all of them by the bounds, read
         * the counters back only when the bounds pass the capacity (then
         * with room for several more batches like this one) */
        if (D->d.cap == 0 || D->ub_codes + n_logical > D->d.codes_cap || 2 * (D->ub_codes + n_logical) > D->d.cap ||
            D->ub_used + chars_ub > D->d.arena_cap) {
            const int64_t f = n_logical <= ((int64_t)1 << 20) ? 8 : 2;
            dict_read(D);
            dict_reserve(D, f * n_logical, f * chars_ub);
            D->ub_codes = (int64_t)D->h_ctr[VG_DICT_CODES];
            D->ub_used = (int64_t)D->h_ctr[VG_DICT_USED];
        }
        D->ub_codes += n_logical;
        D->ub_used += chars_ub;
    } else if (insert) {
        vg_dmemset(D->d_ctr + VG_DICT_ROWS, 0, 16);
        vg_check_rc(vgk_dict_prepass(c, d_sel, n_logical, D->d_ctr, vg_stream()), "string dictionary");
        dict_read(D);
        dict_reserve(D, (int64_t)D->h_ctr[VG_DICT_ROWS], (int64_t)D->h_ctr[VG_DICT_BYTES]);
        D->ub_codes = (int64_t)D->h_ctr[VG_DICT_CODES] + (int64_t)D->h_ctr[VG_DICT_ROWS];
        D->ub_used = (int64_t)D->h_ctr[VG_DICT_USED] + (int64_t)D->h_ctr[VG_DICT_BYTES];
    } else if (D->d.cap == 0) {
        dict_reserve(D, 0, 0);
    }
    vg_check_rc(vgk_dict_encode(&D->d, c, d_sel, n_logical, insert, d_codes, err_word(D), vg_stream()),
                "string dictionary");
}

int64_t vg_dict_size(VgDict *D) {
    dict_read(D);
    return (int64_t)D->h_ctr[VG_DICT_CODES];
}

const VgStrDict *vg_dict_device(VgDict *D) { return &D->d; }

/* The strings' order: perm[r] = the code of rank r, rank[code] = r (both
 * device arrays the caller frees).  A stable sort of the codes by columns
 * of 8-byte big-endian chunks and the length, whose lexicographic order is
 * memcmp order with the shorter string first on a common prefix -- the
 * reference's string order (src/sort.c:32-116 through the same compare as
 * src/scalar_ops.c:78-107). */
void vg_dict_order(VgDict *D, int32_t **d_perm, int64_t **d_rank) {
    const int64_t n = vg_dict_size(D);
    *d_perm = (int32_t *)vg_dmalloc(a256((size_t)(n ? n : 1) * 4));
    *d_rank = (int64_t *)vg_dmalloc(a256((size_t)(n ? n : 1) * 8));
    if (n == 0) return;
    const int64_t maxlen = (int64_t)D->h_ctr[VG_DICT_MAXLEN];
    const int n_chunks = (int)((maxlen + 7) / 8);
    const int nk = n_chunks + 1;
    int64_t *chunks = (int64_t *)vg_dmalloc(a256((size_t)nk * (size_t)n * 8));
    vg_check_rc(vgk_dict_chunks(&D->d, n, n_chunks, chunks, vg_stream()), "string order");
    VgCol *cols = (VgCol *)vg_xcalloc((size_t)nk, sizeof(VgCol));
    int *kc = (int *)vg_xcalloc((size_t)nk, sizeof(int));
    int *kd = (int *)vg_xcalloc((size_t)nk, sizeof(int));
    for (int k = 0; k < nk; k++) {
        cols[k].type = VEC_INT64;
        cols[k].data = chunks + (size_t)k * (size_t)n;
        kc[k] = k;
    }
    const size_t sb = vgk_sort_rows_scratch(n);
    void *work = vg_dmalloc(sb);
    vg_check_rc(vgk_sort_rows(cols, kc, kd, nk, *d_perm, n, work, sb, vg_stream()), "string order");
    vg_check_rc(vgk_rank_of(*d_perm, n, *d_rank, vg_stream()), "string order");
    vg_dfree(work);
    vg_dfree(chunks);
    free(cols);
    free(kc);
    free(kd);
}

/* A string column of n rows from codes (through perm when given), NA where
 * the validity word bit is clear. */
VecArray vg_dict_strings(VgDict *D, const int64_t *d_codes, const uint32_t *d_valid, const int32_t *d_perm,
                         int64_t n) {
    VgStrView *views = (VgStrView *)vg_dmalloc(a256((size_t)(n ? n : 1) * 16));
    vg_check_rc(vgk_dict_views(&D->d, d_codes, d_valid, d_perm, n, views, vg_stream()), "string keys");
    VgCol c;
    memset(&c, 0, sizeof(c));
    c.type = VEC_STRING;
    c.data = views;
    c.valid = d_valid;
    VecArray a = vg_download_strings(&c, NULL, n);
    vg_dfree(views);
    return a;
}
