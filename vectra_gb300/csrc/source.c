/*
 * source.c -- a table as a source node.  For any consumer it behaves like
 * the reference's ScanNode (src/scan.c:107-127): each next_batch returns a
 * malloc-owned copy of the next batch_rows rows.  libvgpu nodes instead pull
 * batches straight onto the device: in place for device-resident tables
 * and for mapped page-locked host tables (the kernels read host memory),
 * by asynchronous copies for other host tables.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "vg_host.h"

typedef struct {
    VecNode base;
    int n_cols;
    int flags;
    int64_t n_rows, batch_rows, cursor;
    void **data;
    uint8_t **validity;
    int *types;
} VgSource;

static VecBatch *source_next(VecNode *self);
static void source_free(VecNode *self);

int vg_is_table_source(const VecNode *n) { return n && n->next_batch == source_next; }

static size_t elem(int type) { return type == VEC_BOOL ? 1 : 8; }

/* dst bits [0, n) = src bits [off, off + n) (reference bitmap order) */
static void copy_bits(uint8_t *dst, const uint8_t *src, int64_t off, int64_t n) {
    if ((off & 7) == 0) {
        memcpy(dst, src + off / 8, (size_t)vg_vbytes(n));
        return;
    }
    memset(dst, 0, (size_t)vg_vbytes(n));
    for (int64_t i = 0; i < n; i++) {
        int64_t s = off + i;
        if ((src[s >> 3] >> (s & 7)) & 1) dst[i >> 3] |= (uint8_t)(1u << (i & 7));
    }
}

static VecBatch *source_next(VecNode *self) {
    VgSource *s = (VgSource *)self;
    if (s->cursor >= s->n_rows) return NULL;
    int64_t lo = s->cursor, n = s->n_rows - lo;
    if (n > s->batch_rows) n = s->batch_rows;
    s->cursor += n;
    VecBatch *b = vg_batch_alloc(s->n_cols, n);
    for (int c = 0; c < s->n_cols; c++) {
        VecArray a;
        memset(&a, 0, sizeof(a));
        a.type = (VecType)s->types[c];
        a.length = n;
        a.owns_data = 1;
        a.validity = (uint8_t *)vg_xcalloc((size_t)vg_vbytes(n), 1);
        void *v = vg_xcalloc((size_t)n * elem(a.type) + 1, 1);
        if (a.type == VEC_BOOL) a.buf.bln = (uint8_t *)v; else a.buf.i64 = (int64_t *)v;
        const char *src = (const char *)s->data[c] + (size_t)lo * elem(a.type);
        const uint8_t *vsrc = s->validity[c];
        if (s->flags & VGPU_SRC_DEVICE) {
            vg_d2h(v, src, (size_t)n * elem(a.type));
            if (vsrc) {
                int64_t b0 = lo / 8, nb = (lo + n + 7) / 8 - b0;
                uint8_t *tmp = (uint8_t *)vg_xmalloc((size_t)nb);
                vg_d2h(tmp, vsrc + b0, (size_t)nb);
                vg_sync();
                copy_bits(a.validity, tmp, lo & 7, n);
                free(tmp);
            }
            vg_sync();
        } else {
            memcpy(v, src, (size_t)n * elem(a.type));
            if (vsrc) copy_bits(a.validity, vsrc, lo, n);
        }
        if (!vsrc) memset(a.validity, 0xFF, (size_t)vg_vbytes(n));
        /* bits past the last row stay clear */
        if (n & 7) a.validity[n / 8] &= (uint8_t)((1u << (n & 7)) - 1);
        b->columns[c] = a;
        b->col_names[c] = vg_xstrdup(self->output_schema.col_names[c]);
    }
    return b;
}

int vg_source_pull(VecNode *n, const uint8_t *need, VgDBatch *out) {
    VgSource *s = (VgSource *)n;
    memset(out, 0, sizeof(*out));
    if (s->cursor >= s->n_rows) return 0;
    int64_t lo = s->cursor, rows = s->n_rows - lo;
    if (rows > s->batch_rows) rows = s->batch_rows;
    s->cursor += rows;
    out->n_rows = rows;
    out->n_cols = s->n_cols;
    out->row_base = lo;
    out->cols = (VgCol *)vg_xcalloc((size_t)s->n_cols, sizeof(VgCol));
    if (s->flags & (VGPU_SRC_DEVICE | VGPU_SRC_MAPPED)) {
        /* in place; validity bitmaps are 4-byte aligned, row lo sits at bit
         * lo%32 of word lo/32 */
        out->in_host = (s->flags & VGPU_SRC_MAPPED) != 0;
        for (int c = 0; c < s->n_cols; c++) {
            out->cols[c].type = s->types[c];
            out->cols[c].data = (const char *)s->data[c] + (size_t)lo * elem(s->types[c]);
            out->cols[c].valid = s->validity[c] ? (const uint32_t *)(s->validity[c] + (lo >> 5) * 4) : NULL;
            out->cols[c].voff = (int32_t)(lo & 31);
        }
        return 1;
    }
    size_t total = 0;
    for (int c = 0; c < s->n_cols; c++)
        if (!need || need[c])
            total += (((size_t)rows * elem(s->types[c]) + 255) & ~(size_t)255) +
                     ((((size_t)(rows + 31) / 32) * 4 + 4 + 255) & ~(size_t)255);
    char *blk = total ? (char *)vg_dmalloc(total) : NULL;
    out->block = blk;
    size_t off = 0;
    for (int c = 0; c < s->n_cols; c++) {
        out->cols[c].type = s->types[c];
        if (need && !need[c]) continue;
        size_t vb = (size_t)rows * elem(s->types[c]);
        char *dv = blk + off;
        off += (vb + 255) & ~(size_t)255;
        vg_h2d(dv, (const char *)s->data[c] + (size_t)lo * elem(s->types[c]), vb);
        out->cols[c].data = dv;
        size_t wb = ((size_t)(rows + 31) / 32) * 4 + 4;
        char *dm = blk + off;
        off += (wb + 255) & ~(size_t)255;
        if (s->validity[c]) {
            /* the bytes holding rows [lo, lo+rows), starting at the 4-byte
             * word of row lo; never past the end of the host bitmap */
            int64_t b0 = (lo >> 5) * 4;
            int64_t b1 = (lo + rows + 7) / 8;
            vg_dmemset(dm, 0, wb);
            vg_h2d(dm, s->validity[c] + b0, (size_t)(b1 - b0));
            out->cols[c].valid = (const uint32_t *)dm;
            out->cols[c].voff = (int32_t)(lo & 31);
        }
    }
    return 1;
}

static void source_free(VecNode *self) {
    VgSource *s = (VgSource *)self;
    if (!(s->flags & (VGPU_SRC_BORROW | VGPU_SRC_DEVICE | VGPU_SRC_MAPPED))) {
        for (int c = 0; c < s->n_cols; c++) {
            free(s->data[c]);
            free(s->validity[c]);
        }
    }
    free(s->data);
    free(s->validity);
    free(s->types);
    vg_schema_free(&self->output_schema);
    free(s);
}

VecNode *vgpu_table_source_create(int n_cols, const char *const *names, const int *types,
                                  const void *const *data, const uint8_t *const *validity,
                                  int64_t n_rows, int64_t batch_rows, int flags) {
    /* selection vectors and filter row ids are int32 (src/types.h:70-85), so
     * a batch holds at most INT32_MAX rows; the default (whole table in one
     * batch) is clamped to that */
    if (batch_rows <= 0) batch_rows = n_rows > 0 ? (n_rows > VGPU_MAX_BATCH_ROWS ? VGPU_MAX_BATCH_ROWS : n_rows) : 1;
    if (n_cols <= 0 || n_rows < 0) { vg_set_error("table source: bad shape"); return NULL; }
    if (batch_rows > VGPU_MAX_BATCH_ROWS) {
        vg_set_error("table source: batch_rows %lld is above the largest batch, %lld rows", (long long)batch_rows,
                     (long long)VGPU_MAX_BATCH_ROWS);
        return NULL;
    }
    for (int c = 0; c < n_cols; c++) {
        if (types[c] != VEC_INT64 && types[c] != VEC_DOUBLE && types[c] != VEC_BOOL) {
            vg_set_error("table source: column '%s' has a type the GPU path does not support", names[c]);
            return NULL;
        }
    }
    if (flags & VGPU_SRC_MAPPED) {
        /* every buffer must be host memory the device addresses directly */
        for (int c = 0; c < n_cols; c++) {
            const void *bufs[2] = {data[c], validity ? validity[c] : NULL};
            for (int b = 0; b < 2; b++) {
                if (!bufs[b]) continue;
                struct cudaPointerAttributes a;
                memset(&a, 0, sizeof(a));
                if (cudaPointerGetAttributes(&a, bufs[b]) != cudaSuccess || a.type != cudaMemoryTypeHost ||
                    a.devicePointer != bufs[b]) {
                    cudaGetLastError();
                    vg_set_error("table source: column '%s' is not page-locked host memory the device can "
                                 "address in place", names[c]);
                    return NULL;
                }
                if (b == 1 && ((uintptr_t)bufs[b] & 3)) {
                    vg_set_error("table source: validity of column '%s' is not 4-byte aligned", names[c]);
                    return NULL;
                }
            }
        }
    }
    VgSource *s = (VgSource *)vg_xcalloc(1, sizeof(VgSource));
    s->n_cols = n_cols;
    s->flags = flags;
    s->n_rows = n_rows;
    s->batch_rows = batch_rows;
    s->data = (void **)vg_xcalloc((size_t)n_cols, sizeof(void *));
    s->validity = (uint8_t **)vg_xcalloc((size_t)n_cols, sizeof(uint8_t *));
    s->types = (int *)vg_xcalloc((size_t)n_cols, sizeof(int));
    VecType *ts = (VecType *)vg_xcalloc((size_t)n_cols, sizeof(VecType));
    for (int c = 0; c < n_cols; c++) {
        s->types[c] = types[c];
        ts[c] = (VecType)types[c];
        if (flags & (VGPU_SRC_BORROW | VGPU_SRC_DEVICE | VGPU_SRC_MAPPED)) {
            s->data[c] = (void *)data[c];
            s->validity[c] = validity ? (uint8_t *)validity[c] : NULL;
        } else {
            size_t vb = (size_t)n_rows * elem(types[c]);
            s->data[c] = vg_xmalloc(vb);
            memcpy(s->data[c], data[c], vb);
            if (validity && validity[c]) {
                s->validity[c] = (uint8_t *)vg_xmalloc((size_t)vg_vbytes(n_rows));
                memcpy(s->validity[c], validity[c], (size_t)vg_vbytes(n_rows));
            }
        }
    }
    s->base.output_schema = vg_schema_make(n_cols, (char *const *)names, ts);
    free(ts);
    s->base.next_batch = source_next;
    s->base.free_node = source_free;
    /* not "ScanNode": the reference optimizer casts nodes of that kind to its
     * ScanNode struct and reads the .vtr file header through it
     * (src/optimize.c:38-41, 90-91, 360-363); an unknown kind stops its
     * propagation there (src/optimize.c:343) */
    s->base.kind = "VgpuTableSource";
    return &s->base;
}
