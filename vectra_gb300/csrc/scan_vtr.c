/*
 * scan_vtr.c -- the .vtr scan node (replaces src/scan.c; reads the format of
 * src/vtr1.c:39-392 with code of its own).
 *
 * scan_node_create returns a node whose struct prefix is the reference's
 * ScanNode {base, file, col_mask, next_rg, predicate, pred_borrowed} and
 * whose file handle starts with Vtr1File {fp, header, rowgroups}, with the
 * kind "ScanNode": the optimizer prunes col_mask and the output schema and
 * attaches a FilterNode's predicate through those fields
 * (src/optimize.c:38-77, 356-371), exactly as on the reference's node.
 *
 * Two ways out of the node:
 *  - next_batch (any consumer): the next row group that the pushed-down
 *    predicate does not rule out, as a malloc-owned batch of the selected
 *    columns, as vtr1_read_rowgroup returns it (src/vtr1.c:306-392);
 *  - vg_scan_pull (libvgpu nodes): the same row group's needed columns read
 *    with pread straight into a page-locked staging block laid out like the
 *    device block, then one asynchronous copy to the device.  A pool of
 *    reader threads reads the next row groups ahead, each into a staging
 *    block of its own (a ring of up to 32), while the caller hands the
 *    groups that are ready to the device in file order; a block is reused
 *    only after the event recorded behind its copy has completed.  The
 *    readers only read the file: every CUDA call and every error report
 *    stays on the calling thread.  VGPU_SCAN_THREADS sets the number of
 *    readers (0: the caller reads each group itself, with two blocks).
 *
 * Row-group pruning restates predicate_might_match (src/scan.c:12-105):
 * AND / OR of `column <op> numeric literal` terms against the row group's
 * v3 min / max statistics (valid values only), anything else may match.
 */
#define _GNU_SOURCE
#include <errno.h>
#include <fcntl.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include <cuda_runtime_api.h>

#include "vg_host.h"

typedef struct {
    Vtr1File f;                 /* reference prefix */
    int fd;                     /* pread handle (same file) */
    int n_cols;
    int64_t *valid_off;         /* [rg * n_cols + c]: file offset of the validity bitmap */
    int64_t *str_len;           /* [rg * n_cols + c]: string data bytes (string columns) */
} VgVtrFile;

enum { PF_FREE = 0, PF_QUEUED, PF_READY, PF_FAILED };
#define VG_SCAN_RING 32
#define VG_SCAN_MAX_READERS 16

/* one row group read ahead into a page-locked staging block */
typedef struct {
    int64_t g;                  /* row group */
    int state;                  /* PF_*, under the pool's mutex */
    int err;                    /* errno of a failed read (0: short file) */
    char *h;                    /* page-locked staging block */
    size_t cap;
    cudaEvent_t ev;             /* recorded behind the block's copy */
    int ev_live;
    int copy_pending;
} VgPre;

typedef struct {
    ScanNode sn;                /* reference prefix */
    int64_t rows_out;           /* rows emitted so far (stream position) */
    /* read-ahead (device path) */
    int pf_on;
    uint8_t *pf_need;           /* per output column: read for the device */
    uint32_t pf_rg;             /* next row group to consider for reading ahead */
    int n_slots, head, count;   /* ring: slots head .. head+count-1 hold groups in file order */
    VgPre slot[VG_SCAN_RING];
    int n_readers;
    pthread_t th[VG_SCAN_MAX_READERS];
    pthread_mutex_t mu;
    pthread_cond_t cv_task, cv_done;
    int q[VG_SCAN_RING];        /* slots waiting for a reader */
    int q_head, q_n;
    int stop;
} VgScan;

static VecBatch *scan_next(VecNode *self);
static void scan_free(VecNode *self);

int vg_is_vtr_scan(const VecNode *n) { return n && n->next_batch == scan_next; }

/* ---- file ---------------------------------------------------------- */

static void rd(FILE *fp, void *p, size_t n, const char *what) {
    if (n && fread(p, 1, n, fp) != n) vg_fail("unexpected end of file reading %s", what);
}

static void pread_all(int fd, void *dst, size_t n, int64_t off) {
    char *p = (char *)dst;
    while (n > 0) {
        ssize_t r = pread(fd, p, n, (off_t)off);
        if (r <= 0) vg_fail("unexpected end of file reading column data");
        p += r;
        n -= (size_t)r;
        off += r;
    }
}

static int64_t data_bytes(int type, int64_t n) {
    return type == VEC_BOOL ? n : 8 * n;
}

static void vtr_close(VgVtrFile *v) {
    if (!v) return;
    if (v->f.fp) fclose(v->f.fp);
    if (v->fd >= 0) close(v->fd);
    vg_schema_free(&v->f.header.schema);
    if (v->f.rowgroups) {
        for (uint32_t g = 0; g < v->f.header.n_rowgroups; g++) free(v->f.rowgroups[g].col_stats);
        free(v->f.rowgroups);
    }
    free(v->valid_off);
    free(v->str_len);
    free(v);
}

/* Header (magic "VTR1", version 1-3, columns with their names, types and,
 * from version 2, annotations), then the row-group index: each group's
 * offset, row count, v3 statistics and the offsets of its columns. */
static VgVtrFile *vtr_open(const char *path) {
    FILE *fp = fopen(path, "rb");
    if (!fp) vg_fail("cannot open file: %s", path);
    char magic[4];
    if (fread(magic, 1, 4, fp) != 4 || memcmp(magic, "VTR1", 4) != 0) {
        fclose(fp);
        vg_fail("not a valid .vtr file (bad magic): %s", path);
    }
    VgVtrFile *v = (VgVtrFile *)vg_xcalloc(1, sizeof(VgVtrFile));
    v->f.fp = fp;
    v->fd = -1;
    uint16_t ver = 0, nc = 0;
    rd(fp, &ver, 2, "the version");
    if (ver < 1 || ver > 3) {
        vtr_close(v);
        vg_fail("unsupported .vtr version: %u", (unsigned)ver);
    }
    v->f.header.version = ver;
    rd(fp, &nc, 2, "the column count");
    char **names = (char **)vg_xcalloc(nc ? nc : 1, sizeof(char *));
    char **ann = (char **)vg_xcalloc(nc ? nc : 1, sizeof(char *));
    VecType *types = (VecType *)vg_xcalloc(nc ? nc : 1, sizeof(VecType));
    for (int c = 0; c < nc; c++) {
        uint16_t len = 0;
        rd(fp, &len, 2, "a column name");
        names[c] = (char *)vg_xmalloc((size_t)len + 1);
        rd(fp, names[c], len, "a column name");
        names[c][len] = 0;
        uint8_t t = 0;
        rd(fp, &t, 1, "a column type");
        types[c] = (VecType)t;
        if (ver >= 2) {
            uint16_t al = 0;
            rd(fp, &al, 2, "an annotation");
            if (al) {
                ann[c] = (char *)vg_xmalloc((size_t)al + 1);
                rd(fp, ann[c], al, "an annotation");
                ann[c][al] = 0;
            }
        }
    }
    v->f.header.schema = vg_schema_make(nc, names, types);
    for (int c = 0; c < nc; c++) {
        v->f.header.schema.col_annotations[c] = ann[c];
        free(names[c]);
    }
    free(names);
    free(ann);
    free(types);
    v->n_cols = nc;
    uint32_t nrg = 0;
    rd(fp, &nrg, 4, "the row-group count");
    v->f.header.n_rowgroups = nrg;
    v->f.rowgroups = (Vtr1RowGroup *)vg_xcalloc(nrg ? nrg : 1, sizeof(Vtr1RowGroup));
    v->valid_off = (int64_t *)vg_xcalloc((size_t)(nrg ? nrg : 1) * (nc ? nc : 1), sizeof(int64_t));
    v->str_len = (int64_t *)vg_xcalloc((size_t)(nrg ? nrg : 1) * (nc ? nc : 1), sizeof(int64_t));
    int64_t pos = ftell(fp);
    for (uint32_t g = 0; g < nrg; g++) {
        Vtr1RowGroup *rg = &v->f.rowgroups[g];
        rg->file_offset = pos;
        if (fseek(fp, (long)pos, SEEK_SET) != 0) vg_fail("unexpected end of file");
        uint64_t n = 0;
        rd(fp, &n, 8, "a row count");
        rg->n_rows = (int64_t)n;
        pos += 8;
        if (ver >= 3) {
            rg->col_stats = (Vtr1ColStat *)vg_xcalloc(nc ? nc : 1, sizeof(Vtr1ColStat));
            for (int c = 0; c < nc; c++) {
                uint8_t has = 0;
                uint64_t a = 0, b = 0;
                rd(fp, &has, 1, "statistics");
                rd(fp, &a, 8, "statistics");
                rd(fp, &b, 8, "statistics");
                Vtr1ColStat *st = &rg->col_stats[c];
                st->has_stats = has;
                if (!has) continue;
                if (v->f.header.schema.col_types[c] == VEC_BOOL) {
                    st->bln.min = (uint8_t)a;
                    st->bln.max = (uint8_t)b;
                } else {
                    memcpy(&st->i64.min, &a, 8);   /* int64 and double share the bytes */
                    memcpy(&st->i64.max, &b, 8);
                }
            }
            pos += 17 * (int64_t)nc;
        }
        for (int c = 0; c < nc; c++) {
            const int t = v->f.header.schema.col_types[c];
            v->valid_off[(size_t)g * nc + c] = pos;
            pos += vg_vbytes((int64_t)n);
            if (t == VEC_STRING) {
                pos += 8 * ((int64_t)n + 1);
                uint64_t dl = 0;
                if (fseek(fp, (long)pos, SEEK_SET) != 0) vg_fail("unexpected end of file");
                rd(fp, &dl, 8, "string data length");
                v->str_len[(size_t)g * nc + c] = (int64_t)dl;
                pos += 8 + (int64_t)dl;
            } else {
                pos += data_bytes(t, (int64_t)n);
            }
        }
    }
    v->fd = open(path, O_RDONLY | O_CLOEXEC);
    if (v->fd < 0) {
        vtr_close(v);
        vg_fail("cannot open file: %s", path);
    }
    return v;
}

/* ---- pruning (src/scan.c:12-105) ------------------------------------ */

static int might_match(const VecExpr *p, const Vtr1ColStat *stats, const VecSchema *s) {
    if (!p || !stats) return 1;
    if (p->kind == EXPR_BOOL && p->op == '&') return might_match(p->left, stats, s) && might_match(p->right, stats, s);
    if (p->kind == EXPR_BOOL && p->op == '|') return might_match(p->left, stats, s) || might_match(p->right, stats, s);
    if (p->kind != EXPR_CMP) return 1;
    const VecExpr *c = NULL, *l = NULL;
    int col_left = 0;
    const int lit_r = p->right->kind == EXPR_LIT_INT64 || p->right->kind == EXPR_LIT_DOUBLE;
    const int lit_l = p->left->kind == EXPR_LIT_INT64 || p->left->kind == EXPR_LIT_DOUBLE;
    if (p->left->kind == EXPR_COL_REF && lit_r) {
        c = p->left;
        l = p->right;
        col_left = 1;
    } else if (p->right->kind == EXPR_COL_REF && lit_l) {
        c = p->right;
        l = p->left;
    } else {
        return 1;
    }
    const int ci = vg_schema_find(s, c->col_name);
    if (ci < 0 || !stats[ci].has_stats) return 1;
    const double lit = l->kind == EXPR_LIT_DOUBLE ? l->lit_dbl : (double)l->lit_i64;
    double lo, hi;
    if (s->col_types[ci] == VEC_INT64) {
        lo = (double)stats[ci].i64.min;
        hi = (double)stats[ci].i64.max;
    } else if (s->col_types[ci] == VEC_DOUBLE) {
        lo = stats[ci].dbl.min;
        hi = stats[ci].dbl.max;
    } else {
        return 1;
    }
    char op = p->op;
    const char op2 = p->op2;
    /* `literal op column`: < and > swap sides (the second character stays) */
    if (!col_left) op = op == '<' ? '>' : op == '>' ? '<' : op;
    if (op == '>' && op2 == ' ') return hi > lit;
    if (op == '>' && op2 == '=') return hi >= lit;
    if (op == '<' && op2 == ' ') return lo < lit;
    if (op == '<' && op2 == '=') return lo <= lit;
    if (op == '=' && op2 == '=') return lo <= lit && hi >= lit;
    if (op == '!' && op2 == '=') return !(lo == lit && hi == lit);
    return 1;
}

/* the next row group the pushed-down predicate does not rule out, or -1 */
static int64_t next_group(VgScan *s) {
    VgVtrFile *v = (VgVtrFile *)s->sn.file;
    while (s->sn.next_rg < v->f.header.n_rowgroups) {
        const uint32_t g = s->sn.next_rg++;
        if (s->sn.predicate && v->f.header.version >= 3 &&
            !might_match(s->sn.predicate, v->f.rowgroups[g].col_stats, &v->f.header.schema))
            continue;
        return g;
    }
    return -1;
}

/* ---- host batches (src/vtr1.c:306-392) ------------------------------- */

static void reset_ahead(VgScan *s);

static VecBatch *scan_next(VecNode *self) {
    VgScan *s = (VgScan *)self;
    VgVtrFile *v = (VgVtrFile *)s->sn.file;
    if (s->pf_on) reset_ahead(s);    /* groups read ahead for the device are read again here */
    const int64_t g = next_group(s);
    if (g < 0) return NULL;
    const int64_t n = v->f.rowgroups[g].n_rows;
    int n_sel = 0;
    for (int c = 0; c < v->n_cols; c++) n_sel += s->sn.col_mask[c] != 0;
    VecBatch *b = vg_batch_alloc(n_sel, n);
    int o = 0;
    for (int c = 0; c < v->n_cols; c++) {
        if (!s->sn.col_mask[c]) continue;
        const int t = v->f.header.schema.col_types[c];
        VecArray a;
        memset(&a, 0, sizeof(a));
        a.type = (VecType)t;
        a.length = n;
        a.owns_data = 1;
        a.validity = (uint8_t *)vg_xcalloc((size_t)(vg_vbytes(n) ? vg_vbytes(n) : 1), 1);
        int64_t off = v->valid_off[(size_t)g * v->n_cols + c];
        pread_all(v->fd, a.validity, (size_t)vg_vbytes(n), off);
        off += vg_vbytes(n);
        if (t == VEC_STRING) {
            a.buf.str.offsets = (int64_t *)vg_xcalloc((size_t)n + 1, 8);
            pread_all(v->fd, a.buf.str.offsets, 8 * ((size_t)n + 1), off);
            const int64_t dl = v->str_len[(size_t)g * v->n_cols + c];
            a.buf.str.data_len = dl;
            a.buf.str.data = dl ? (char *)vg_xmalloc((size_t)dl) : NULL;
            pread_all(v->fd, a.buf.str.data, (size_t)dl, off + 8 * (n + 1) + 8);
        } else {
            void *d = vg_xcalloc((size_t)(n ? data_bytes(t, n) : 1), 1);
            pread_all(v->fd, d, (size_t)data_bytes(t, n), off);
            if (t == VEC_BOOL) a.buf.bln = (uint8_t *)d;
            else a.buf.i64 = (int64_t *)d;
        }
        b->columns[o] = a;
        b->col_names[o] = vg_xstrdup(v->f.header.schema.col_names[c]);
        o++;
    }
    s->rows_out += n;
    return b;
}

/* ---- device batches -------------------------------------------------- */

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

/* pread of n bytes at off without reporting: 0, or the errno of a failed
 * read (-1: the file ends early) */
static int pread_quiet(int fd, void *dst, size_t n, int64_t off) {
    char *p = (char *)dst;
    while (n > 0) {
        ssize_t r = pread(fd, p, n, (off_t)off);
        if (r < 0 && errno == EINTR) continue;
        if (r <= 0) return r < 0 ? errno : -1;
        p += r;
        n -= (size_t)r;
        off += r;
    }
    return 0;
}

/* A column's part of row group g's staging / device block: its values
 * (for strings one 16-byte view per row, made on the device), its
 * validity words, and for strings the file's offsets and characters. */
static size_t col_bytes(const VgVtrFile *v, int64_t g, int c, int64_t n) {
    const size_t vwords = (size_t)((n + 31) / 32) * 4;
    const int t = v->f.header.schema.col_types[c];
    if (t != VEC_STRING) return a256((size_t)data_bytes(t, n)) + a256(vwords);
    const int64_t dl = v->str_len[(size_t)g * v->n_cols + c];
    return a256((size_t)n * 16) + a256(vwords) + a256(8 * ((size_t)n + 1)) + a256((size_t)dl + 1);
}

/* bytes of row group g's staging / device block for the needed columns,
 * each part 256-byte aligned */
static size_t group_bytes(const VgScan *s, int64_t g, const uint8_t *need) {
    const VgVtrFile *v = (const VgVtrFile *)s->sn.file;
    const int64_t n = v->f.rowgroups[g].n_rows;
    size_t total = 0;
    int o = 0;
    for (int c = 0; c < v->n_cols; c++) {
        if (!s->sn.col_mask[c]) continue;
        if (need[o]) total += col_bytes(v, g, c, n);
        o++;
    }
    return total;
}

/* reads row group g's needed columns into h in the device block's layout;
 * 0 or an error as pread_quiet */
static int read_group(const VgScan *s, int64_t g, const uint8_t *need, char *h) {
    const VgVtrFile *v = (const VgVtrFile *)s->sn.file;
    const int64_t n = v->f.rowgroups[g].n_rows;
    const size_t vwords = (size_t)((n + 31) / 32) * 4;
    size_t off = 0;
    int o = 0;
    for (int c = 0; c < v->n_cols; c++) {
        if (!s->sn.col_mask[c]) continue;
        const int t = v->f.header.schema.col_types[c];
        if (need[o] && t == VEC_STRING) {
            /* views (made on the device), validity, offsets, characters */
            const int64_t fo = v->valid_off[(size_t)g * v->n_cols + c];
            const int64_t dl = v->str_len[(size_t)g * v->n_cols + c];
            const size_t ov = off + a256((size_t)n * 16), oo = ov + a256(vwords), oc = oo + a256(8 * ((size_t)n + 1));
            if (vg_vbytes(n) & 3) memset(h + ov + ((size_t)vg_vbytes(n) & ~(size_t)3), 0, 4);
            int e = pread_quiet(v->fd, h + ov, (size_t)vg_vbytes(n), fo);
            if (!e) e = pread_quiet(v->fd, h + oo, 8 * ((size_t)n + 1), fo + vg_vbytes(n));
            if (!e) e = pread_quiet(v->fd, h + oc, (size_t)dl, fo + vg_vbytes(n) + 8 * (n + 1) + 8);
            if (e) return e;
            off += col_bytes(v, g, c, n);
        } else if (need[o]) {
            const int64_t fo = v->valid_off[(size_t)g * v->n_cols + c];
            const size_t db = (size_t)data_bytes(t, n);
            int e = pread_quiet(v->fd, h + off, db, fo + vg_vbytes(n));
            if (e) return e;
            off += a256(db);
            if (vg_vbytes(n) & 3)   /* the last 32-bit word's bytes past the bitmap read as 0 */
                memset(h + off + ((size_t)vg_vbytes(n) & ~(size_t)3), 0, 4);
            e = pread_quiet(v->fd, h + off, (size_t)vg_vbytes(n), fo);
            if (e) return e;
            off += a256(vwords);
        }
        o++;
    }
    return 0;
}

static void *reader_main(void *arg) {
    VgScan *s = (VgScan *)arg;
    pthread_mutex_lock(&s->mu);
    for (;;) {
        while (!s->stop && s->q_n == 0) pthread_cond_wait(&s->cv_task, &s->mu);
        if (s->stop) break;
        const int i = s->q[s->q_head];
        s->q_head = (s->q_head + 1) % VG_SCAN_RING;
        s->q_n--;
        VgPre *p = &s->slot[i];
        const int64_t g = p->g;
        char *h = p->h;
        pthread_mutex_unlock(&s->mu);
        const int e = read_group(s, g, s->pf_need, h);
        pthread_mutex_lock(&s->mu);
        p->err = e;
        p->state = e ? PF_FAILED : PF_READY;
        pthread_cond_broadcast(&s->cv_done);
    }
    pthread_mutex_unlock(&s->mu);
    return NULL;
}

/* the next row group after pf_rg that the pushed-down predicate does not
 * rule out (advancing pf_rg), or -1 */
static int64_t next_ahead(VgScan *s) {
    VgVtrFile *v = (VgVtrFile *)s->sn.file;
    while (s->pf_rg < v->f.header.n_rowgroups) {
        const uint32_t g = s->pf_rg++;
        if (s->sn.predicate && v->f.header.version >= 3 &&
            !might_match(s->sn.predicate, v->f.rowgroups[g].col_stats, &v->f.header.schema))
            continue;
        return g;
    }
    return -1;
}

/* waits for every queued read (the caller holds no lock) */
static void drain_reads(VgScan *s) {
    if (s->n_readers == 0) return;
    pthread_mutex_lock(&s->mu);
    for (int k = 0; k < s->count; k++) {
        VgPre *p = &s->slot[(s->head + k) % s->n_slots];
        while (p->state == PF_QUEUED) pthread_cond_wait(&s->cv_done, &s->mu);
    }
    pthread_mutex_unlock(&s->mu);
}

/* forgets the groups read ahead (the next pull starts from the delivered
 * position again) */
static void reset_ahead(VgScan *s) {
    drain_reads(s);
    for (int k = 0; k < s->count; k++) s->slot[(s->head + k) % s->n_slots].state = PF_FREE;
    s->head = 0;
    s->count = 0;
    s->pf_rg = s->sn.next_rg;
}

static void start_readers(VgScan *s) {
    int nr = 8;
    const long cpus = sysconf(_SC_NPROCESSORS_ONLN);
    if (cpus > 0 && cpus < nr) nr = (int)cpus;
    const char *env = getenv("VGPU_SCAN_THREADS");
    if (env) nr = atoi(env);
    if (nr < 0) nr = 0;
    if (nr > VG_SCAN_MAX_READERS) nr = VG_SCAN_MAX_READERS;
    s->n_slots = nr == 0 ? 2 : (2 * nr < VG_SCAN_RING ? 2 * nr : VG_SCAN_RING);
    if (pthread_mutex_init(&s->mu, NULL) != 0 || pthread_cond_init(&s->cv_task, NULL) != 0 ||
        pthread_cond_init(&s->cv_done, NULL) != 0)
        vg_fail("scan: reader pool could not be set up");
    s->n_readers = 0;
    for (int i = 0; i < nr; i++) {
        if (pthread_create(&s->th[i], NULL, reader_main, s) != 0) break;
        s->n_readers++;
    }
    if (nr > 0 && s->n_readers == 0) s->n_slots = 2;   /* no thread could start: read on the caller */
}

/* fills the ring with the next row groups and queues their reads */
static void fill_ahead(VgScan *s) {
    while (s->count < s->n_slots) {
        const int i = (s->head + s->count) % s->n_slots;
        VgPre *p = &s->slot[i];
        if (p->copy_pending) {
            /* the block's previous copy must have read it; while other
             * groups are queued, a copy still running ends the filling
             * instead of a wait */
            cudaError_t e = cudaEventQuery(p->ev);
            if (e == cudaErrorNotReady) {
                if (s->count > 0) return;
                e = cudaEventSynchronize(p->ev);
            }
            if (e != cudaSuccess) vg_fail("scan: staging copy failed: %s", cudaGetErrorString(e));
            p->copy_pending = 0;
        }
        const int64_t g = next_ahead(s);
        if (g < 0) return;
        const size_t bytes = group_bytes(s, g, s->pf_need);
        if (p->cap < bytes) {
            if (p->h) cudaFreeHost(p->h);
            p->h = NULL;
            p->cap = 0;
            const size_t want = bytes + bytes / 4;
            if (cudaHostAlloc((void **)&p->h, want, cudaHostAllocDefault) != cudaSuccess) {
                cudaGetLastError();
                p->h = NULL;
                s->pf_rg--;          /* this group is not taken */
                vg_fail("scan: page-locked staging block of %zu bytes could not be allocated", want);
            }
            p->cap = want;
        }
        p->g = g;
        p->err = 0;
        s->count++;
        if (s->n_readers == 0) {
            p->state = PF_READY;     /* read when it is taken */
            continue;
        }
        pthread_mutex_lock(&s->mu);
        p->state = PF_QUEUED;
        s->q[(s->q_head + s->q_n) % VG_SCAN_RING] = i;
        s->q_n++;
        pthread_cond_signal(&s->cv_task);
        pthread_mutex_unlock(&s->mu);
    }
}

int vg_scan_pull(VecNode *node, const uint8_t *need, VgDBatch *out) {
    VgScan *s = (VgScan *)node;
    VgVtrFile *v = (VgVtrFile *)s->sn.file;
    memset(out, 0, sizeof(*out));
    int n_sel = 0;
    for (int c = 0; c < v->n_cols; c++) n_sel += s->sn.col_mask[c] != 0;
    /* the columns this consumer needs */
    uint8_t *nd = (uint8_t *)vg_xcalloc((size_t)(n_sel ? n_sel : 1), 1);
    int o = 0;
    for (int c = 0; c < v->n_cols; c++) {
        if (!s->sn.col_mask[c]) continue;
        nd[o] = (uint8_t)(!need || need[o]);
        o++;
    }
    if (!s->pf_on) {
        start_readers(s);
        s->pf_on = 1;
        s->pf_need = nd;
        s->pf_rg = s->sn.next_rg;
    } else if (memcmp(nd, s->pf_need, (size_t)(n_sel ? n_sel : 1)) != 0) {
        reset_ahead(s);              /* another set of columns: read again from here */
        free(s->pf_need);
        s->pf_need = nd;
    } else {
        free(nd);
    }
    fill_ahead(s);
    if (s->count == 0) return 0;
    VgPre *p = &s->slot[s->head];
    if (s->n_readers > 0) {
        pthread_mutex_lock(&s->mu);
        while (p->state == PF_QUEUED) pthread_cond_wait(&s->cv_done, &s->mu);
        pthread_mutex_unlock(&s->mu);
    } else {
        p->err = read_group(s, p->g, s->pf_need, p->h);
        if (p->err) p->state = PF_FAILED;
    }
    const int64_t g = p->g;
    s->head = (s->head + 1) % s->n_slots;
    s->count--;
    s->sn.next_rg = (uint32_t)g + 1;
    if (p->state == PF_FAILED) {
        const int e = p->err;
        p->state = PF_FREE;
        reset_ahead(s);
        if (e > 0) vg_fail("scan: reading column data failed: %s", strerror(e));
        vg_fail("unexpected end of file reading column data");
    }
    p->state = PF_FREE;

    const int64_t n = v->f.rowgroups[g].n_rows;
    out->n_rows = n;
    out->n_cols = n_sel;
    out->row_base = s->rows_out;
    out->cols = (VgCol *)vg_xcalloc((size_t)(n_sel ? n_sel : 1), sizeof(VgCol));
    s->rows_out += n;
    const size_t total = group_bytes(s, g, s->pf_need);
    o = 0;
    for (int c = 0; c < v->n_cols; c++) {
        if (!s->sn.col_mask[c]) continue;
        out->cols[o].type = v->f.header.schema.col_types[c];
        o++;
    }
    if (total == 0) {
        fill_ahead(s);
        return 1;
    }
    char *d = (char *)vg_dmalloc(total);
    out->block = d;
    const size_t vwords = (size_t)((n + 31) / 32) * 4;
    size_t off = 0;
    o = 0;
    for (int c = 0; c < v->n_cols; c++) {
        if (!s->sn.col_mask[c]) continue;
        const int t = v->f.header.schema.col_types[c];
        if (s->pf_need[o]) {
            const size_t cb = col_bytes(v, g, c, n);
            out->cols[o].data = d + off;
            off += t == VEC_STRING ? a256((size_t)n * 16) : a256((size_t)data_bytes(t, n));
            out->cols[o].valid = (const uint32_t *)(d + off);
            out->cols[o].voff = 0;
            if (t == VEC_STRING) {
                if (!out->str_chars) out->str_chars = (int64_t *)vg_xcalloc((size_t)(n_sel ? n_sel : 1), sizeof(int64_t));
                out->str_chars[o] = v->str_len[(size_t)g * v->n_cols + c];
                /* the file's offsets drive the device's reads: they must
                 * start at 0 or above, never decrease, stay within the
                 * characters and give values below 2 GiB */
                const int64_t *fo = (const int64_t *)(p->h + off + a256(vwords));
                const int64_t dl = v->str_len[(size_t)g * v->n_cols + c];
                int bad = n > 0 && (fo[0] < 0 || fo[n] > dl);
                for (int64_t i = 0; i < n && !bad; i++)
                    bad = fo[i + 1] < fo[i] || fo[i + 1] - fo[i] > (int64_t)0x7FFFFFFF;
                if (bad) {
                    vg_dbatch_release(out);
                    vg_fail("scan: malformed string offsets in column '%s'", v->f.header.schema.col_names[c]);
                }
            }
            off = (size_t)((char *)out->cols[o].data - d) + cb;
        }
        o++;
    }
    cudaStream_t st = (cudaStream_t)vg_stream();
    cudaError_t e = cudaMemcpyAsync(d, p->h, total, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !p->ev_live) {
        e = cudaEventCreateWithFlags(&p->ev, cudaEventDisableTiming);
        if (e == cudaSuccess) p->ev_live = 1;
    }
    if (e == cudaSuccess) e = cudaEventRecord(p->ev, st);
    if (e != cudaSuccess) {
        vg_dbatch_release(out);
        vg_fail("scan: copy of a row group to the device failed: %s", cudaGetErrorString(e));
    }
    p->copy_pending = 1;
    /* string columns: views over the copied offsets and characters */
    o = 0;
    for (int c = 0; c < v->n_cols; c++) {
        if (!s->sn.col_mask[c]) continue;
        if (s->pf_need[o] && v->f.header.schema.col_types[c] == VEC_STRING && n > 0) {
            const char *views = (const char *)out->cols[o].data;
            const char *offs = views + a256((size_t)n * 16) + a256(vwords);
            const char *chars = offs + a256(8 * ((size_t)n + 1));
            vg_check_rc(vgk_str_views((const int64_t *)offs, 0, chars, n, (VgStrView *)views, vg_stream()),
                        "string column upload");
        }
        o++;
    }
    fill_ahead(s);                   /* keep the readers busy while this group is used */
    return 1;
}

/* ---- node ------------------------------------------------------------ */

static void scan_free(VecNode *self) {
    VgScan *s = (VgScan *)self;
    if (s->pf_on) {
        if (s->n_readers > 0) {
            pthread_mutex_lock(&s->mu);
            s->stop = 1;
            pthread_cond_broadcast(&s->cv_task);
            pthread_mutex_unlock(&s->mu);
            for (int i = 0; i < s->n_readers; i++) pthread_join(s->th[i], NULL);
        }
        pthread_mutex_destroy(&s->mu);
        pthread_cond_destroy(&s->cv_task);
        pthread_cond_destroy(&s->cv_done);
        for (int i = 0; i < VG_SCAN_RING; i++) {
            VgPre *p = &s->slot[i];
            if (p->ev_live) {
                cudaEventSynchronize(p->ev);
                cudaEventDestroy(p->ev);
            }
            if (p->h) cudaFreeHost(p->h);
        }
        free(s->pf_need);
    }
    if (s->sn.predicate && !s->sn.pred_borrowed) vg_expr_free(s->sn.predicate);
    vtr_close((VgVtrFile *)s->sn.file);
    free(s->sn.col_mask);
    vg_schema_free(&s->sn.base.output_schema);
    free(s);
}

ScanNode *scan_node_create(const char *path, int *col_indices, int n_selected) {
    VgVtrFile *v = vtr_open(path);
    VgScan *s = (VgScan *)vg_xcalloc(1, sizeof(VgScan));
    s->sn.file = &v->f;
    const VecSchema *fs = &v->f.header.schema;
    s->sn.col_mask = (int *)vg_xcalloc((size_t)(fs->n_cols ? fs->n_cols : 1), sizeof(int));
    if (!col_indices) {
        for (int c = 0; c < fs->n_cols; c++) s->sn.col_mask[c] = 1;
        s->sn.base.output_schema = vg_schema_copy(fs);
    } else {
        for (int i = 0; i < n_selected; i++) {
            if (col_indices[i] < 0 || col_indices[i] >= fs->n_cols) {
                const int bad = col_indices[i];
                vtr_close(v);
                free(s->sn.col_mask);
                free(s);
                vg_fail("column index out of range: %d", bad);
            }
            s->sn.col_mask[col_indices[i]] = 1;
        }
        int k = 0;
        for (int c = 0; c < fs->n_cols; c++) k += s->sn.col_mask[c];
        char **names = (char **)vg_xcalloc((size_t)(k ? k : 1), sizeof(char *));
        VecType *types = (VecType *)vg_xcalloc((size_t)(k ? k : 1), sizeof(VecType));
        int j = 0;
        for (int c = 0; c < fs->n_cols; c++) {
            if (!s->sn.col_mask[c]) continue;
            names[j] = fs->col_names[c];
            types[j] = fs->col_types[c];
            j++;
        }
        s->sn.base.output_schema = vg_schema_make(k, names, types);
        free(names);
        free(types);
    }
    s->sn.base.next_batch = scan_next;
    s->sn.base.free_node = scan_free;
    s->sn.base.kind = "ScanNode";
    return &s->sn;
}
