/*
 * runtime.c -- libvgpu runtime: errors, device memory and stream, host
 * batch helpers, and moving batches between host and device.
 */
#define _GNU_SOURCE
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <stdatomic.h>
#include <time.h>
#include <unistd.h>
#include <cuda_runtime_api.h>

#include "vg_host.h"

extern unsigned long long vg_launch_counter;

/* ------------------------------------------------------------------ */
/* errors                                                              */
/* ------------------------------------------------------------------ */

static char g_msg[1024];
static jmp_buf *g_jmp = NULL;
static long g_warnings = 0;

const char *vgpu_last_error(void) { return g_msg; }
long vgpu_warning_count(void) { return g_warnings; }
void vg_warn_count(long n) { g_warnings += n; }
unsigned long long vgpu_kernel_launches(void) { return vg_launch_counter; }

/* The reference engine's error entry point (src/error.c:4-11).  When libvgpu
 * is linked into the vectra package, the engine's own definition (which
 * raises an R error) takes precedence over this weak one. */
__attribute__((weak)) void vectra_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    snprintf(g_msg, sizeof(g_msg), "%s", buf);
    if (g_jmp) longjmp(*g_jmp, 1);
    fprintf(stderr, "libvgpu: %s\n", g_msg);
    abort();
}

void vg_set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
}

static void sync_before_error(void);

static void release_scope(void);

void vg_fail(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
    sync_before_error();
    release_scope();
    vectra_error("%s", g_msg);
    abort();   /* vectra_error does not return */
}

const char *vgk_last_cuda_error(void);
const char *vgk_agg_last_error(void);
const char *vgk_join_last_error(void);
const char *vgk_sort_last_error(void);

void vg_check_rc(int rc, const char *what) {
    if (rc == 0) return;
    const char *m = vgk_last_cuda_error();
    if (!m || !*m) m = vgk_agg_last_error();
    if (!m || !*m) m = vgk_join_last_error();
    if (!m || !*m) m = vgk_sort_last_error();
    if (!m || !*m) m = vgk_pagg_last_error();
    if (!m || !*m) m = vgk_jit_error();
    if (!m || !*m) m = vgk_str_last_error();
    vg_fail("%s failed: %s", what, (m && *m) ? m : "unknown device error");
}

/* ------------------------------------------------------------------ */
/* device, stream, memory                                              */
/* ------------------------------------------------------------------ */

static int g_inited = 0;
static int g_device = 0;
static cudaStream_t g_own_stream = NULL;
static cudaStream_t g_user_stream = NULL;
static int g_use_user = 0;

int vgpu_init(int device) {
    if (g_inited) return 0;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        snprintf(g_msg, sizeof(g_msg), "libvgpu: no CUDA device available");
        return -1;
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        snprintf(g_msg, sizeof(g_msg), "libvgpu: cannot select device %d", device);
        return -1;
    }
    struct cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) == cudaSuccess && p.major < 10) {
        snprintf(g_msg, sizeof(g_msg), "libvgpu: device %d is sm_%d%d; sm_103 required",
                 device, p.major, p.minor);
        return -1;
    }
    if (cudaStreamCreateWithFlags(&g_own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        snprintf(g_msg, sizeof(g_msg), "libvgpu: stream creation failed");
        return -1;
    }
    /* keep freed device memory cached in the default pool */
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    g_device = device;
    g_inited = 1;
    return 0;
}

/* Before an error leaves the library, the failed call's kernels and copies
 * on the library's stream end (a device that has faulted answers at once
 * with its error, which is ignored here: the message is already set). */
static void sync_before_error(void) {
    if (g_inited) (void)cudaStreamSynchronize(g_use_user ? g_user_stream : g_own_stream);
}

void vg_ensure_init(void) {
    if (!g_inited && vgpu_init(0) != 0) vg_fail("%s", g_msg);
}

void vgpu_set_stream(void *s) {
    g_user_stream = (cudaStream_t)s;
    g_use_user = (s != NULL);
}

void *vgpu_get_stream(void) { return (void *)vg_stream(); }

vg_stream_t vg_stream(void) {
    vg_ensure_init();
    return (vg_stream_t)(g_use_user ? g_user_stream : g_own_stream);
}

/* The stream for work that must not initialise the library (the
 * allocation-free entry point): the caller's stream if one was set, else
 * the library's own once it exists and belongs to the current device, else
 * the legacy default stream (of whichever device is current). */
vg_stream_t vg_stream_noinit(void) {
    if (g_use_user) return (vg_stream_t)g_user_stream;
    if (!g_inited) return (vg_stream_t)0;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != g_device) {
        cudaGetLastError();
        return (vg_stream_t)0;
    }
    return (vg_stream_t)g_own_stream;
}

int vgpu_synchronize(void) {
    if (!g_inited) return 0;
    return cudaStreamSynchronize((cudaStream_t)vg_stream()) == cudaSuccess ? 0 : -1;
}

/* ---- the per-call scope of temporary device memory --------------------
 * Every device allocation made inside a node API call (next_batch of a
 * libvgpu node, entered through vg_scope_enter / vg_scope_leave) is
 * recorded until it is freed.  A call that fails releases what is still
 * recorded -- after the stream has synchronised, before vectra_error -- so
 * a failed query leaves no device memory behind; state a node keeps
 * across calls (join tables, kept batches) is allocated with
 * vg_dmalloc_kept and released by the node's free_node.  The reference's
 * contract: release device and pinned memory, then raise
 * (src/error.c:4-11). */
static void **g_tmp = NULL;
static size_t g_tmp_n = 0, g_tmp_cap = 0;
static int g_scope_depth = 0;
static long g_alloc_seq = 0;          /* device allocations so far (fault injection) */
static long g_fail_at = -1;           /* VGPU_FAIL_ALLOC: the allocation that fails */

void vg_scope_enter(void) { g_scope_depth++; }

void vg_scope_leave(void) {
    if (--g_scope_depth <= 0) {
        g_scope_depth = 0;
        g_tmp_n = 0;
    }
}

static void tmp_add(void *p) {
    if (g_scope_depth <= 0 || !p) return;
    if (g_tmp_n == g_tmp_cap) {
        size_t nc = g_tmp_cap ? 2 * g_tmp_cap : 64;
        void **q = (void **)realloc(g_tmp, nc * sizeof(void *));
        if (!q) return;   /* not recorded: at worst not released on an error */
        g_tmp = q;
        g_tmp_cap = nc;
    }
    g_tmp[g_tmp_n++] = p;
}

static void tmp_remove(void *p) {
    for (size_t i = g_tmp_n; i-- > 0;) {
        if (g_tmp[i] == p) {
            g_tmp[i] = g_tmp[--g_tmp_n];
            return;
        }
    }
}

/* after the stream has synchronised: the failed call's temporaries */
static void release_scope(void) {
    if (g_inited)
        for (size_t i = 0; i < g_tmp_n; i++) cudaFreeAsync(g_tmp[i], g_use_user ? g_user_stream : g_own_stream);
    g_tmp_n = 0;
    g_scope_depth = 0;
}

static void *dmalloc_raw(size_t bytes) {
    void *p = NULL;
    if (bytes == 0) bytes = 256;
    if (g_fail_at == -1) {
        const char *e = getenv("VGPU_FAIL_ALLOC");
        g_fail_at = e ? atol(e) : 0;
    }
    cudaError_t e = (g_fail_at > 0 && ++g_alloc_seq == g_fail_at)
                        ? cudaErrorMemoryAllocation
                        : cudaMallocAsync(&p, bytes, (cudaStream_t)vg_stream());
    if (e != cudaSuccess) vg_fail("device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    return p;
}

void *vg_dmalloc(size_t bytes) {
    void *p = dmalloc_raw(bytes);
    tmp_add(p);
    return p;
}

void *vg_dmalloc_kept(size_t bytes) { return dmalloc_raw(bytes); }

void vg_dkeep(void *p) {
    if (p) tmp_remove(p);
}

void vg_dfree(void *p) {
    if (!p) return;
    tmp_remove(p);
    cudaFreeAsync(p, (cudaStream_t)vg_stream());
}

/* Fault injection for tests: the n-th device allocation from now fails
 * (0: none). */
void vgpu_debug_fail_alloc(long n) {
    g_alloc_seq = 0;
    g_fail_at = n > 0 ? n : 0;
}

int vgk_wait_selftest(long long limit, uint32_t *code, vg_stream_t s);

/* The device's bounded wait run out on purpose: a kernel polls, through the
 * group table's own wait, a word that nothing changes, for `limit` polls;
 * the expired wait comes back as an error (-1, vgpu_last_error), the device
 * stays usable.  0 would mean the wait ended, which it cannot. */
int vgpu_wait_selftest(long long limit) {
    vg_ensure_init();
    uint32_t code = 0;
    if (vgk_wait_selftest(limit, &code, vg_stream()) != 0) {
        vg_set_error("wait self-test: %s", vgk_agg_last_error());
        return -1;
    }
    if (code & VG_ERR_WAIT) {
        vg_set_error("a bounded wait on the device expired after %lld polls (error code %u)", limit, code);
        return -1;
    }
    return 0;
}

/* Bytes the device's default memory pool has handed out and not taken
 * back (the pool libvgpu allocates from), or -1. */
long long vgpu_device_bytes_in_use(void) {
    int dev = 0;
    cudaMemPool_t pool;
    unsigned long long v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess ||
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &v) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return (long long)v;
}

void vg_h2d(void *dst, const void *src, size_t bytes) {
    if (!bytes) return;
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)vg_stream());
    if (e != cudaSuccess) vg_fail("host to device copy failed: %s", cudaGetErrorString(e));
}

void vg_d2h(void *dst, const void *src, size_t bytes) {
    if (!bytes) return;
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)vg_stream());
    if (e != cudaSuccess) vg_fail("device to host copy failed: %s", cudaGetErrorString(e));
}

/* A second stream for result copies that overlap device work on the main
 * stream: vg_copy_after_main() makes it wait for everything queued on the
 * main stream so far; vg_d2h_copy() copies on it (into pageable memory the
 * call returns when the copy is done). */
static cudaStream_t g_copy_stream = NULL;

static cudaStream_t copy_stream(void) {
    if (!g_copy_stream) {
        cudaError_t e = cudaStreamCreateWithFlags(&g_copy_stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) vg_fail("copy stream: %s", cudaGetErrorString(e));
    }
    return g_copy_stream;
}

void vg_copy_after_main(void) {
    cudaEvent_t ev;
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ev, (cudaStream_t)vg_stream());
    if (e == cudaSuccess) e = cudaStreamWaitEvent(copy_stream(), ev, 0);
    if (e != cudaSuccess) vg_fail("copy stream ordering: %s", cudaGetErrorString(e));
    cudaEventDestroy(ev);
}

void vg_d2h_copy(void *dst, const void *src, size_t bytes) {
    if (!bytes) return;
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, copy_stream());
    if (e != cudaSuccess) vg_fail("device to host copy failed: %s", cudaGetErrorString(e));
}

void vg_copy_sync(void) {
    if (!g_copy_stream) return;
    cudaError_t e = cudaStreamSynchronize(g_copy_stream);
    if (e != cudaSuccess) vg_fail("copy stream: %s", cudaGetErrorString(e));
}

/* A host column over values already on the host (malloc-owned, taken
 * over) with its validity copied from the device bitmap d_valid. */
VecArray vg_host_column(int type, int64_t n, void *values, const uint32_t *d_valid) {
    VecArray a;
    memset(&a, 0, sizeof(a));
    a.type = (VecType)type;
    a.length = n;
    a.owns_data = 1;
    a.validity = (uint8_t *)vg_xcalloc((size_t)vg_vbytes(n), 1);
    if (type == VEC_BOOL) a.buf.bln = (uint8_t *)values;
    else a.buf.i64 = (int64_t *)values;
    if (n > 0) vg_d2h(a.validity, d_valid, (size_t)vg_vbytes(n));
    return a;
}

void vg_dmemset(void *dst, int v, size_t bytes) {
    if (!bytes) return;
    cudaError_t e = cudaMemsetAsync(dst, v, bytes, (cudaStream_t)vg_stream());
    if (e != cudaSuccess) vg_fail("device memset failed: %s", cudaGetErrorString(e));
}

void vg_sync(void) {
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)vg_stream());
    if (e != cudaSuccess) vg_fail("device execution failed: %s", cudaGetErrorString(e));
}

static void *g_pin = NULL;
static size_t g_pin_bytes = 0;

/* 256 page-locked bytes of status words, apart from the scratch above (a
 * status copy can stay in flight while the scratch is regrown) */
static void *g_stat_pin = NULL;
uint32_t *vg_pinned_status(void) {
    if (!g_stat_pin) {
        cudaError_t e = cudaMallocHost(&g_stat_pin, 256);
        if (e != cudaSuccess) {
            g_stat_pin = NULL;
            vg_fail("page-locked allocation of 256 bytes failed: %s", cudaGetErrorString(e));
        }
    }
    return (uint32_t *)g_stat_pin;
}

void *vg_pinned_scratch(size_t bytes) {
    if (bytes <= g_pin_bytes) return g_pin;
    size_t nb = 65536;
    while (nb < bytes) nb <<= 1;
    if (g_pin) {
        vg_sync();                      /* no copy into the old buffer is in flight */
        cudaFreeHost(g_pin);
        g_pin = NULL;
        g_pin_bytes = 0;
    }
    cudaError_t e = cudaMallocHost(&g_pin, nb);
    if (e != cudaSuccess) {
        g_pin = NULL;
        vg_fail("page-locked allocation of %zu bytes failed: %s", nb, cudaGetErrorString(e));
    }
    g_pin_bytes = nb;
    return g_pin;
}

/* ------------------------------------------------------------------ */
/* host memory, batches, schemas                                       */
/* ------------------------------------------------------------------ */

void *vg_xmalloc(size_t n) {
    void *p = malloc(n ? n : 1);
    if (!p) vg_fail("host allocation of %zu bytes failed", n);
    return p;
}
void *vg_xcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s ? s : 1);
    if (!p) vg_fail("host allocation failed");
    return p;
}
char *vg_xstrdup(const char *s) {
    size_t n = strlen(s) + 1;
    char *p = (char *)vg_xmalloc(n);
    memcpy(p, s, n);
    return p;
}

VecBatch *vg_batch_alloc(int n_cols, int64_t n_rows) {
    VecBatch *b = (VecBatch *)vg_xcalloc(1, sizeof(VecBatch));
    b->n_cols = n_cols;
    b->n_rows = n_rows;
    b->columns = (VecArray *)vg_xcalloc((size_t)n_cols, sizeof(VecArray));
    b->col_names = (char **)vg_xcalloc((size_t)n_cols, sizeof(char *));
    return b;
}

/* frees a batch exactly as the reference's vec_batch_free does
 * (src/batch.c:19-29, src/array.c:41-58) */
void vg_batch_free(VecBatch *b) {
    if (!b) return;
    for (int i = 0; i < b->n_cols; i++) {
        VecArray *a = &b->columns[i];
        free(a->validity);
        switch (a->type) {
        case VEC_INT64: free(a->buf.i64); break;
        case VEC_DOUBLE: free(a->buf.dbl); break;
        case VEC_BOOL: free(a->buf.bln); break;
        case VEC_STRING:
            free(a->buf.str.offsets);
            if (a->owns_data) free(a->buf.str.data);
            break;
        }
        free(b->col_names[i]);
    }
    free(b->columns);
    free(b->col_names);
    free(b->sel);
    free(b);
}

void vgpu_batch_free(VecBatch *b) { vg_batch_free(b); }

VecSchema vg_schema_make(int n, char *const *names, const VecType *types) {
    VecSchema s;
    s.n_cols = n;
    s.col_names = (char **)vg_xcalloc((size_t)n, sizeof(char *));
    s.col_types = (VecType *)vg_xcalloc((size_t)n, sizeof(VecType));
    s.col_annotations = (char **)vg_xcalloc((size_t)n, sizeof(char *));
    for (int i = 0; i < n; i++) {
        s.col_names[i] = vg_xstrdup(names[i]);
        s.col_types[i] = types[i];
    }
    return s;
}

VecSchema vg_schema_copy(const VecSchema *src) {
    VecSchema s = vg_schema_make(src->n_cols, src->col_names, src->col_types);
    for (int i = 0; i < src->n_cols; i++)
        if (src->col_annotations && src->col_annotations[i])
            s.col_annotations[i] = vg_xstrdup(src->col_annotations[i]);
    return s;
}

void vg_schema_free(VecSchema *s) {
    for (int i = 0; i < s->n_cols; i++) {
        free(s->col_names[i]);
        if (s->col_annotations) free(s->col_annotations[i]);
    }
    free(s->col_names);
    free(s->col_types);
    free(s->col_annotations);
    memset(s, 0, sizeof(*s));
}

int vg_schema_find(const VecSchema *s, const char *name) {
    for (int i = 0; i < s->n_cols; i++)
        if (strcmp(s->col_names[i], name) == 0) return i;
    return -1;
}

/* ------------------------------------------------------------------ */
/* host <-> device batches                                             */
/* ------------------------------------------------------------------ */

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

static size_t value_bytes(int type, int64_t n) {
    return (size_t)n * (type == VEC_BOOL ? 1 : 8);
}
static size_t valid_bytes_dev(int64_t n) { return (size_t)((n + 31) / 32) * 4; }

/* Two page-locked staging blocks for batches of foreign children (host
 * batches the caller frees): a batch's needed columns are copied into one
 * block laid out like its device block, then moved by one asynchronous copy;
 * the host batch is freed at once and the block is reused only after the
 * event behind its copy has completed, so copy and kernels overlap the
 * child's production of the next batch. */
static void *g_stage[2];
static size_t g_stage_bytes[2];
static cudaEvent_t g_stage_ev[2];
static int g_stage_ev_live[2];
static int g_stage_cur;

static char *stage_take(size_t bytes) {
    const int i = g_stage_cur;
    if (g_stage_ev_live[i]) {
        cudaError_t e = cudaEventSynchronize(g_stage_ev[i]);
        if (e != cudaSuccess) vg_fail("staging copy failed: %s", cudaGetErrorString(e));
    }
    if (g_stage_bytes[i] < bytes) {
        if (g_stage[i]) cudaFreeHost(g_stage[i]);
        g_stage[i] = NULL;
        g_stage_bytes[i] = 0;
        size_t want = bytes + bytes / 4;
        if (cudaHostAlloc(&g_stage[i], want, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            vg_fail("page-locked staging block of %zu bytes could not be allocated", want);
        }
        g_stage_bytes[i] = want;
    }
    return (char *)g_stage[i];
}

static void stage_send(void *dst, const void *src, size_t bytes) {
    const int i = g_stage_cur;
    cudaStream_t st = (cudaStream_t)vg_stream();
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !g_stage_ev_live[i]) {
        e = cudaEventCreateWithFlags(&g_stage_ev[i], cudaEventDisableTiming);
        if (e == cudaSuccess) g_stage_ev_live[i] = 1;
    }
    if (e == cudaSuccess) e = cudaEventRecord(g_stage_ev[i], st);
    if (e != cudaSuccess) vg_fail("staged copy to the device failed: %s", cudaGetErrorString(e));
    g_stage_cur ^= 1;
}

/* bytes of a string column's characters in one batch (below 4 GiB: a
 * device view holds a 32-bit length) */
static size_t str_bytes(const VecArray *a, int64_t n) {
    if (n <= 0) return 0;
    const int64_t e = a->buf.str.offsets[n];
    if (e < 0 || e > (int64_t)0xFFFFFFFFll)
        vg_fail("string column: %lld bytes in one batch; the GPU path takes less than 4 GiB per batch", (long long)e);
    return (size_t)e;
}

/* the device reads each row's bytes through its offsets: they must start
 * at 0 or above and never decrease */
static void check_offsets(const VecArray *a, int64_t n) {
    const int64_t *o = a->buf.str.offsets;
    if (n <= 0) return;
    if (!o || o[0] < 0 || (o[n] > 0 && !a->buf.str.data)) vg_fail("string column: malformed offsets");
    for (int64_t i = 0; i < n; i++) {
        if (o[i + 1] < o[i]) vg_fail("string column: offsets decrease at row %lld", (long long)i);
        if (o[i + 1] - o[i] > (int64_t)0x7FFFFFFF)
            vg_fail("string column: a value of %lld bytes (the GPU path takes below 2 GiB)",
                    (long long)(o[i + 1] - o[i]));
    }
}

/* A needed column's part of the device block: values (for strings, one
 * 16-byte view per row), validity words, and for strings the offsets and
 * the characters, from which the views are made on the device. */
static size_t col_dev_bytes(const VecArray *a, int64_t n) {
    if (a->type == VEC_STRING)
        return a256((size_t)n * 16) + a256(valid_bytes_dev(n)) + a256((size_t)(n + 1) * 8) + a256(str_bytes(a, n) + 1);
    return a256(value_bytes(a->type, n)) + a256(valid_bytes_dev(n));
}

int vg_pull(VecNode *child, const uint8_t *need, int keep_host, VgDBatch *out) {
    memset(out, 0, sizeof(*out));
    if (vg_is_table_source(child) && !keep_host) return vg_source_pull(child, need, out);
    if (vg_is_vtr_scan(child) && !keep_host) return vg_scan_pull(child, need, out);
    VecBatch *b = child->next_batch(child);
    if (!b) return 0;
    int64_t n = b->n_rows;
    out->n_rows = n;
    out->n_cols = b->n_cols;
    out->cols = (VgCol *)vg_xcalloc((size_t)b->n_cols, sizeof(VgCol));
    size_t total = 0;
    for (int c = 0; c < b->n_cols; c++) {
        if (!need || !need[c]) continue;
        total += col_dev_bytes(&b->columns[c], n);
    }
    if (b->sel) total += a256((size_t)b->sel_n * 4);
    char *blk = total ? (char *)vg_dmalloc(total) : NULL;
    out->block = blk;
    /* string columns: where their offsets and characters land, for the
     * views made once the copies are queued */
    int n_str = 0;
    for (int c = 0; c < b->n_cols; c++) n_str += (!need || need[c]) && b->columns[c].type == VEC_STRING;
    size_t *str_at = n_str ? (size_t *)vg_xcalloc((size_t)b->n_cols, sizeof(size_t)) : NULL;
    char *h = (!keep_host && total) ? stage_take(total) : NULL;
    size_t o = 0;
    for (int c = 0; c < b->n_cols; c++) {
        VecArray *a = &b->columns[c];
        out->cols[c].type = a->type;
        if (!need || !need[c]) continue;
        const size_t wb = valid_bytes_dev(n);
        if (a->type == VEC_STRING) {
            /* views, validity, offsets, characters */
            out->cols[c].data = blk + o;
            const size_t ov = o + a256((size_t)n * 16);
            const size_t oo = ov + a256(wb);
            const size_t oc = oo + a256((size_t)(n + 1) * 8);
            const size_t nb = str_bytes(a, n);
            check_offsets(a, n);
            if (n > 0) {
                if (h) {
                    memcpy(h + oo, a->buf.str.offsets, (size_t)(n + 1) * 8);
                    if (nb) memcpy(h + oc, a->buf.str.data, nb);
                } else {
                    vg_h2d(blk + oo, a->buf.str.offsets, (size_t)(n + 1) * 8);
                    vg_h2d(blk + oc, a->buf.str.data, nb);
                }
            }
            str_at[c] = o;
            if (!out->str_chars) out->str_chars = (int64_t *)vg_xcalloc((size_t)b->n_cols, sizeof(int64_t));
            out->str_chars[c] = (int64_t)nb;
            o = ov;
        } else {
            const size_t vb = value_bytes(a->type, n);
            void *src = a->type == VEC_BOOL ? (void *)a->buf.bln : (void *)a->buf.i64;
            if (h) { if (vb) memcpy(h + o, src, vb); }
            else vg_h2d(blk + o, src, vb);
            out->cols[c].data = blk + o;
            o += a256(vb);
        }
        if (a->validity) {
            if (h) {
                memset(h + o + (wb >= 4 ? wb - 4 : 0), 0, wb >= 4 ? 4 : wb);
                memcpy(h + o, a->validity, (size_t)vg_vbytes(n));
            } else {
                if (vg_vbytes(n) & 3) vg_dmemset(blk + o + (vg_vbytes(n) & ~(int64_t)3), 0, 4);
                vg_h2d(blk + o, a->validity, (size_t)vg_vbytes(n));
            }
            out->cols[c].valid = (const uint32_t *)(blk + o);
        }
        o += a256(wb);
        if (a->type == VEC_STRING) o += a256((size_t)(n + 1) * 8) + a256(str_bytes(a, n) + 1);
    }
    if (b->sel) {
        if (h) memcpy(h + o, b->sel, (size_t)b->sel_n * 4);
        else vg_h2d(blk + o, b->sel, (size_t)b->sel_n * 4);
        out->d_sel = (const int32_t *)(blk + o);
        out->sel_n = b->sel_n;
    }
    if (h) stage_send(blk, h, total);
    for (int c = 0; n_str && c < b->n_cols; c++) {
        if ((need && !need[c]) || b->columns[c].type != VEC_STRING) continue;
        const size_t ov = str_at[c] + a256((size_t)n * 16);
        const size_t oo = ov + a256(valid_bytes_dev(n));
        const size_t oc = oo + a256((size_t)(n + 1) * 8);
        vg_check_rc(vgk_str_views((const int64_t *)(blk + oo), 0, blk + oc, n, (VgStrView *)(blk + str_at[c]),
                                  vg_stream()), "string column upload");
    }
    free(str_at);
    if (keep_host) {
        out->host = b;
    } else {
        if (!h) vg_sync();
        vg_batch_free(b);
    }
    return 1;
}

/* Rows [lo, lo + n) of a host column to the device, in one new block
 * (*blk, freed by the caller): values, validity (the bytes holding those
 * rows, so voff = lo % 8), and for strings offsets, characters and views. */
VgCol vg_upload_slice(const VecArray *a, int64_t lo, int64_t n, void **blk) {
    VgCol c;
    memset(&c, 0, sizeof(c));
    c.type = a->type;
    const int64_t b0 = lo / 8, nvb = (lo % 8 + n + 7) / 8;
    const size_t vb = a256((size_t)nvb + 8);
    size_t bytes = vb;
    int64_t s0 = 0, s1 = 0;
    if (a->type == VEC_STRING) {
        s0 = n > 0 ? a->buf.str.offsets[lo] : 0;
        s1 = n > 0 ? a->buf.str.offsets[lo + n] : 0;
        bytes += a256((size_t)n * 16) + a256((size_t)(n + 1) * 8) + a256((size_t)(s1 - s0) + 1);
    } else {
        bytes += a256(value_bytes(a->type, n) + 8);
    }
    char *p = (char *)vg_dmalloc(bytes);
    *blk = p;
    if (n <= 0) return c;
    if (a->validity) {
        vg_dmemset(p, 0, vb);
        vg_h2d(p, a->validity + b0, (size_t)nvb);
        c.valid = (const uint32_t *)p;
        c.voff = (int32_t)(lo % 8);
    }
    char *q = p + vb;
    if (a->type == VEC_STRING) {
        VecArray sl = *a;
        sl.buf.str.offsets = a->buf.str.offsets + lo;
        check_offsets(&sl, n);
        char *views = q, *offs = q + a256((size_t)n * 16), *chars = offs + a256((size_t)(n + 1) * 8);
        vg_h2d(offs, a->buf.str.offsets + lo, (size_t)(n + 1) * 8);
        vg_h2d(chars, a->buf.str.data + s0, (size_t)(s1 - s0));
        vg_check_rc(vgk_str_views((const int64_t *)offs, s0, chars, n, (VgStrView *)views, vg_stream()),
                    "string column upload");
        c.data = views;
    } else {
        const size_t es = a->type == VEC_BOOL ? 1 : 8;
        vg_h2d(q, (const char *)(a->type == VEC_BOOL ? (void *)a->buf.bln : (void *)a->buf.i64) + (size_t)lo * es,
               (size_t)n * es);
        c.data = q;
    }
    return c;
}

/* A device string column (views) -> newly malloc'd host VecArray in the
 * reference's layout, rows d_idx[j] (or j; a negative id gives NA). */
VecArray vg_download_strings(const VgCol *c, const int32_t *d_idx, int64_t n) {
    VecArray a;
    memset(&a, 0, sizeof(a));
    a.type = VEC_STRING;
    a.length = n;
    a.owns_data = 1;
    a.validity = (uint8_t *)vg_xcalloc((size_t)vg_vbytes(n) + 1, 1);
    a.buf.str.offsets = (int64_t *)vg_xcalloc((size_t)n + 1, 8);
    if (n <= 0) {
        a.buf.str.data = (char *)vg_xcalloc(1, 1);
        return a;
    }
    const size_t sb = vgk_scan_scratch(n);
    char *blk = (char *)vg_dmalloc(a256((size_t)n * 4) + a256((size_t)(n + 1) * 8) + a256(valid_bytes_dev(n)) + sb);
    int32_t *len = (int32_t *)blk;
    int64_t *offs = (int64_t *)(blk + a256((size_t)n * 4));
    uint32_t *val = (uint32_t *)((char *)offs + a256((size_t)(n + 1) * 8));
    void *scr = (char *)val + a256(valid_bytes_dev(n));
    vg_check_rc(vgk_str_lengths(c, d_idx, n, len, val, vg_stream()), "string download");
    vg_check_rc(vgk_exclusive_scan(len, n, offs, offs + n, scr, sb, vg_stream()), "string download");
    vg_d2h(a.buf.str.offsets, offs, (size_t)(n + 1) * 8);
    vg_d2h(a.validity, val, (size_t)vg_vbytes(n));
    vg_sync();
    const int64_t total = a.buf.str.offsets[n];
    char *d_chars = (char *)vg_dmalloc((size_t)total + 1);
    vg_check_rc(vgk_str_pack(c, d_idx, n, offs, d_chars, vg_stream()), "string download");
    a.buf.str.data = (char *)vg_xmalloc((size_t)total + 1);
    a.buf.str.data_len = total;
    vg_d2h(a.buf.str.data, d_chars, (size_t)total);
    vg_sync();
    vg_dfree(d_chars);
    vg_dfree(blk);
    return a;
}

void vg_dbatch_release(VgDBatch *b) {
    if (b->block) vg_dfree(b->block);
    if (b->host) vg_batch_free(b->host);
    free(b->cols);
    free(b->str_chars);
    memset(b, 0, sizeof(*b));
}

/* A large fresh host allocation costs the kernel's page zeroing on first
 * touch (about 25 GB/s on one core), several times the copy from the
 * device into touched pages; several threads fault the pages in first. */
typedef struct {
    volatile char *p;
    size_t n, step;
} Touch;

static void *touch_pages(void *arg) {
    Touch *t = (Touch *)arg;
    for (size_t o = 0; o < t->n; o += t->step) t->p[o] = 0;
    return NULL;
}

static void prefault(void *p, size_t n) {
    enum { kMaxThreads = 8 };
    if (n < ((size_t)4 << 20)) return;
    long cpus = sysconf(_SC_NPROCESSORS_ONLN);
    int nt = cpus >= 2 * kMaxThreads ? kMaxThreads : (int)(cpus > 1 ? cpus / 2 : 1);
    if (nt < 2) return;
    long pg = sysconf(_SC_PAGESIZE);
    size_t step = pg > 4096 ? (size_t)pg : 4096;
    size_t chunk = ((n / (size_t)nt) + step - 1) / step * step;
    pthread_t th[kMaxThreads];
    Touch t[kMaxThreads];
    int started = 0;
    for (int i = 0; i < nt; i++) {
        size_t off = (size_t)i * chunk;
        if (off >= n) break;
        t[i].p = (volatile char *)p + off;
        t[i].n = off + chunk <= n ? chunk : n - off;
        t[i].step = step;
        if (pthread_create(&th[i], NULL, touch_pages, &t[i]) != 0) {
            touch_pages(&t[i]);
            continue;
        }
        started |= 1 << i;
    }
    for (int i = 0; i < nt; i++)
        if (started & (1 << i)) pthread_join(th[i], NULL);
}

/* Host buffers faulted in by background threads while the device works
 * (a result whose size is estimated before it is computed). */
/* The buffers are faulted in chunk by chunk in ascending offset (chunk k:
 * bytes [k C, (k + 1) C) of every buffer), chunks handed out to the threads
 * by a counter, so a consumer that fills the buffers from the front can
 * start on the first chunks while the threads are still on later ones. */
struct VgHostBufs {
    int n, nt;
    size_t bytes, chunk, n_chunks;
    void **buf;                    /* the buffers not taken yet */
    void **tbuf;                   /* every buffer, as the threads see them */
    pthread_t th[8];
    int started;
    atomic_size_t next;
    atomic_uchar *done;            /* per chunk */
};

static void *touch_chunks(void *arg) {
    VgHostBufs *h = (VgHostBufs *)arg;
    long pg = sysconf(_SC_PAGESIZE);
    size_t step = pg > 4096 ? (size_t)pg : 4096;
    for (;;) {
        const size_t k = atomic_fetch_add(&h->next, 1);
        if (k >= h->n_chunks) break;
        const size_t lo = k * h->chunk, hi = lo + h->chunk < h->bytes ? lo + h->chunk : h->bytes;
        for (int b = 0; b < h->n; b++)
            for (size_t o = lo; o < hi; o += step) ((volatile char *)h->tbuf[b])[o] = 0;
        atomic_store(&h->done[k], 1);
    }
    return NULL;
}

VgHostBufs *vg_host_bufs_begin(int n, size_t bytes) {
    VgHostBufs *h = (VgHostBufs *)vg_xcalloc(1, sizeof(VgHostBufs));
    h->n = n;
    h->bytes = bytes;
    h->buf = (void **)vg_xcalloc((size_t)n, sizeof(void *));
    h->tbuf = (void **)vg_xcalloc((size_t)n, sizeof(void *));
    for (int b = 0; b < n; b++) {
        h->buf[b] = malloc(bytes ? bytes : 1);
        if (!h->buf[b]) {
            for (int c = 0; c < b; c++) free(h->buf[c]);
            free(h->buf);
            free(h->tbuf);
            free(h);
            return NULL;
        }
        h->tbuf[b] = h->buf[b];
    }
    h->chunk = (size_t)16 << 20;
    h->n_chunks = (bytes + h->chunk - 1) / h->chunk;
    h->done = (atomic_uchar *)vg_xcalloc(h->n_chunks ? h->n_chunks : 1, sizeof(atomic_uchar));
    for (size_t k = 0; k < h->n_chunks; k++) atomic_init(&h->done[k], 0);
    atomic_init(&h->next, 0);
    long cpus = sysconf(_SC_NPROCESSORS_ONLN);
    h->nt = cpus >= 16 ? 8 : (int)(cpus > 1 ? cpus / 2 : 1);
    for (int i = 0; i < h->nt; i++)
        if (pthread_create(&h->th[i], NULL, touch_chunks, h) == 0) h->started |= 1 << i;
    if (!h->started) touch_chunks(h);
    return h;
}

/* Waits until the first `upto` bytes of every buffer are faulted in (the
 * threads always progress: each chunk is finished by the thread that took
 * it). */
void vg_host_bufs_wait_upto(VgHostBufs *h, size_t upto) {
    if (!h) return;
    const size_t kmax = upto >= h->bytes ? h->n_chunks : (upto + h->chunk - 1) / h->chunk;
    for (size_t k = 0; k < kmax; k++)
        while (!atomic_load(&h->done[k])) {
            struct timespec ts = {0, 20000};
            nanosleep(&ts, NULL);
        }
}

/* Waits for the touching threads; the buffers stay with h until taken. */
void vg_host_bufs_wait(VgHostBufs *h) {
    if (!h) return;
    for (int i = 0; i < h->nt; i++)
        if (h->started & (1 << i)) pthread_join(h->th[i], NULL);
    h->started = 0;
}

void *vg_host_bufs_take(VgHostBufs *h, int b, size_t need) {
    if (!h || b >= h->n || need > h->bytes || !h->buf[b]) return NULL;
    void *p = h->buf[b];
    h->buf[b] = NULL;
    return p;
}

void vg_host_bufs_free(VgHostBufs *h) {
    if (!h) return;
    vg_host_bufs_wait(h);
    for (int b = 0; b < h->n; b++) free(h->buf[b]);
    free(h->buf);
    free(h->tbuf);
    free((void *)h->done);
    free(h);
}

VecArray vg_column_from_host(int type, const void *values, const void *valid, int64_t n) {
    VecArray a;
    memset(&a, 0, sizeof(a));
    a.type = (VecType)type;
    a.length = n;
    a.owns_data = 1;
    a.validity = (uint8_t *)vg_xcalloc((size_t)vg_vbytes(n), 1);
    size_t vb = value_bytes(type, n);
    void *dst = vg_xcalloc(vb ? vb : 1, 1);
    if (type == VEC_BOOL) a.buf.bln = (uint8_t *)dst;
    else a.buf.i64 = (int64_t *)dst;
    if (n > 0) {
        memcpy(dst, values, vb);
        if (valid) memcpy(a.validity, valid, (size_t)vg_vbytes(n));
        else memset(a.validity, 0xFF, (size_t)vg_vbytes(n));
    }
    return a;
}

VecArray vg_download_column(int type, const void *d_data, const uint32_t *d_valid, int64_t n) {
    VecArray a;
    memset(&a, 0, sizeof(a));
    a.type = (VecType)type;
    a.length = n;
    a.owns_data = 1;
    a.validity = (uint8_t *)vg_xcalloc((size_t)vg_vbytes(n), 1);
    size_t vb = value_bytes(type, n);
    void *dst = vg_xcalloc(vb ? vb : 1, 1);
    prefault(dst, vb);
    if (type == VEC_BOOL) a.buf.bln = (uint8_t *)dst;
    else a.buf.i64 = (int64_t *)dst;
    if (n > 0) {
        vg_d2h(dst, d_data, vb);
        if (d_valid) vg_d2h(a.validity, d_valid, (size_t)vg_vbytes(n));
        else memset(a.validity, 0xFF, (size_t)vg_vbytes(n));
    }
    return a;
}

/* ------------------------------------------------------------------ */
/* guarded entry points                                                */
/* ------------------------------------------------------------------ */

#define GUARD_BEGIN(T)                                        \
    jmp_buf jb; jmp_buf *prev = g_jmp; g_msg[0] = 0;          \
    if (setjmp(jb)) { g_jmp = prev; return (T)NULL; }         \
    g_jmp = &jb;
#define GUARD_END g_jmp = prev;

VecBatch *vgpu_guard_next_batch(VecNode *node) {
    GUARD_BEGIN(VecBatch *)
    VecBatch *b = node->next_batch(node);
    GUARD_END
    return b;
}
FilterNode *vgpu_guard_filter(VecNode *child, VecExpr *pred) {
    GUARD_BEGIN(FilterNode *)
    FilterNode *r = filter_node_create(child, pred);
    GUARD_END
    return r;
}
ProjectNode *vgpu_guard_project(VecNode *child, int n, ProjEntry *entries) {
    GUARD_BEGIN(ProjectNode *)
    ProjectNode *r = project_node_create(child, n, entries);
    GUARD_END
    return r;
}
GroupAggNode *vgpu_guard_group_agg(VecNode *child, int n_keys, char **key_names, int n_aggs,
                                   AggSpec *specs, const char *temp_dir) {
    GUARD_BEGIN(GroupAggNode *)
    GroupAggNode *r = group_agg_node_create(child, n_keys, key_names, n_aggs, specs, temp_dir);
    GUARD_END
    return r;
}
SortNode *vgpu_guard_sort(VecNode *child, int n_keys, SortKey *keys, const char *temp_dir) {
    GUARD_BEGIN(SortNode *)
    SortNode *r = sort_node_create(child, n_keys, keys, temp_dir);
    GUARD_END
    return r;
}
ScanNode *vgpu_guard_scan(const char *path, int *col_indices, int n_selected) {
    GUARD_BEGIN(ScanNode *)
    ScanNode *r = scan_node_create(path, col_indices, n_selected);
    GUARD_END
    return r;
}
JoinNode *vgpu_guard_join(VecNode *l, VecNode *r, JoinKind kind, int n_keys, JoinKey *keys,
                          const char *sx, const char *sy) {
    GUARD_BEGIN(JoinNode *)
    JoinNode *j = join_node_create(l, r, kind, n_keys, keys, sx, sy);
    GUARD_END
    return j;
}
