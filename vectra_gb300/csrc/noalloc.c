/*
 * noalloc.c -- vgpu_filter_select_static: the filter kernels run over
 * caller-owned device columns with their working space in a fixed
 * device-side array (k_static.cu) instead of allocated memory.
 *
 * Nothing here allocates: no device allocation of any kind and no host
 * heap (the predicate compiles into structs on the stack; the column views
 * are on the stack).  No counterpart in the reference engine; the
 * selection is filter_next_batch's (src/filter.c:13-64).
 */
#include <string.h>

#include "vg_host.h"

int vgk_static_scratch(void **ptr, size_t *bytes);
const char *vgk_static_scratch_error(void);

typedef struct {
    int n;
    const char *const *names;
    const int *types;
} StaticCols;

static int map_static(void *ctx, const char *name, int *type) {
    const StaticCols *c = (const StaticCols *)ctx;
    for (int i = 0; i < c->n; i++) {
        if (c->names[i] && strcmp(c->names[i], name) == 0) {
            *type = c->types[i];
            return i;
        }
    }
    return -1;
}

int vgpu_filter_select_static(int n_cols, const char *const *names, const int *types,
                              const void *const *d_data, const void *const *d_validity,
                              int64_t n_rows, const VecExpr *predicate, int32_t *d_sel_out,
                              int64_t *n_selected) {
    if (!n_selected || !predicate || (n_cols > 0 && (!names || !types || !d_data))) {
        vg_set_error("vgpu_filter_select_static: null argument");
        return -1;
    }
    *n_selected = 0;
    if (n_cols < 0 || n_cols > VG_MAX_COLS) {
        vg_set_error("vgpu_filter_select_static: %d columns (at most %d supported)", n_cols, VG_MAX_COLS);
        return -1;
    }
    if (n_rows < 0 || n_rows > VGPU_STATIC_MAX_ROWS) {
        vg_set_error("vgpu_filter_select_static: %lld rows; at most %lld rows per call "
                     "(the fixed scratch is sized for that)",
                     (long long)n_rows, (long long)VGPU_STATIC_MAX_ROWS);
        return -1;
    }
    if (n_rows > 0 && !d_sel_out) {
        vg_set_error("vgpu_filter_select_static: null selection output");
        return -1;
    }
    VgCol cols[VG_MAX_COLS];
    memset(cols, 0, sizeof(cols));
    for (int i = 0; i < n_cols; i++) {
        if (types[i] != VEC_INT64 && types[i] != VEC_DOUBLE && types[i] != VEC_BOOL) {
            vg_set_error("vgpu_filter_select_static: column %d has an unsupported type", i);
            return -1;
        }
        if (n_rows > 0 && !d_data[i]) {
            vg_set_error("vgpu_filter_select_static: column %d has no data", i);
            return -1;
        }
        if (d_validity && d_validity[i] && ((uintptr_t)d_validity[i] & 3)) {
            vg_set_error("vgpu_filter_select_static: validity bitmap of column %d is not 4-byte aligned", i);
            return -1;
        }
        cols[i].type = types[i];
        cols[i].voff = 0;
        cols[i].data = d_data[i];
        cols[i].valid = d_validity ? (const uint32_t *)d_validity[i] : NULL;
    }
    void *scratch = NULL;
    size_t scratch_bytes = 0;
    if (vgk_static_scratch(&scratch, &scratch_bytes) != 0) {
        vg_set_error("vgpu_filter_select_static: %s", vgk_static_scratch_error());
        return -1;
    }
    if (vgk_filter_scratch_bytes(n_rows) > scratch_bytes) {
        vg_set_error("vgpu_filter_select_static: %lld rows need %zu bytes of scratch, %zu available",
                     (long long)n_rows, vgk_filter_scratch_bytes(n_rows), scratch_bytes);
        return -1;
    }
    StaticCols ctx = {n_cols, names, types};
    VgPred pred;
    VgProg prog;
    int rc;
    int r = vg_compile_pred(predicate, map_static, &ctx, &pred);
    if (r < 0) {
        vg_set_error("vgpu_filter_select_static: %s", vg_compile_error());
        return -1;
    }
    if (r == 1) {
        rc = vgk_filter_pred(cols, n_cols, &pred, n_rows, NULL, 0, d_sel_out, n_selected, scratch,
                             scratch_bytes, vg_stream_noinit());
    } else {
        if (vg_compile_prog(predicate, map_static, &ctx, &prog) != 0) {
            vg_set_error("vgpu_filter_select_static: %s", vg_compile_error());
            return -1;
        }
        if (prog.result_type != VEC_BOOL) {
            vg_set_error("vgpu_filter_select_static: predicate must evaluate to boolean");
            return -1;
        }
        rc = vgk_filter_prog(cols, n_cols, &prog, n_rows, NULL, 0, d_sel_out, n_selected, scratch,
                             scratch_bytes, vg_stream_noinit());
    }
    if (rc != 0) {
        vg_set_error("vgpu_filter_select_static: %s", vgk_last_cuda_error());
        return -1;
    }
    return 0;
}
