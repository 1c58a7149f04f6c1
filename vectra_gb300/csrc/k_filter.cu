// k_filter.cu -- predicate evaluation into selection vectors, general
// expression evaluation and column gathers (sm_103a).
//
// Replaces the reference's per-batch vec_expr_eval + apply_mask_sel
// (src/expr.c:91-281, src/scalar_ops.c:70-203, src/filter.c:13-39):
// instead of materialising one full-length array per sub-expression, each
// warp evaluates 32 logical rows at a time, votes the keep bits into one
// 32-bit word (__ballot_sync) and a second pass turns the words into
// ascending physical row ids with a block-wide prefix sum.

#include <cstdio>
#include <cmath>
#include <cstring>
#include "k_common.cuh"

extern "C" unsigned long long vg_launch_counter = 0;

namespace {

constexpr int kThreads = 256;                 // 8 warps
constexpr int kRowsPerBlock = kThreads * 32;  // one keep word per thread

// ---------------------------------------------------------------------
// keep bit of one row under a conjunction of range terms
// ---------------------------------------------------------------------
VG_DEV bool term_keep(const VgTerm &t, const VgCol *cols, int64_t p) {
    if (t.kind == VG_TERM_NONE) return false;
    const VgCol &c = cols[t.col];
    bool v = vg_valid(c, p);
    if (t.kind == VG_TERM_IS_NA) return !v;
    if (t.kind == VG_TERM_NOT_NA) return v;
    if (!v) return false;
    uint64_t bits = vg_load_bits(c, p);
    int64_t x;
    if (t.domain == VG_DOM_DOUBLE) {
        if (vg_is_nan_bits(bits)) return t.nan_keep != 0;
        x = vg_ord(bits);
    } else {
        x = (int64_t)bits;
    }
    bool in = (x >= t.lo) && (x <= t.hi);
    return t.kind == VG_TERM_RANGE ? in : !in;
}

VG_DEV bool pred_keep(const VgPred &P, const VgCol *cols, int64_t p) {
    for (int i = 0; i < P.n_terms; i++)
        if (!term_keep(P.term[i], cols, p)) return false;
    return true;
}

// ---------------------------------------------------------------------
// postfix program interpreter (one row per lane)
// ---------------------------------------------------------------------
// A cell holds an int64, a double's bits or a bool as 0/1 in v; a string
// as a pointer to its bytes in v and its length in len.
struct Cell { uint64_t v; uint32_t len; bool ok; };

// memcmp over the shorter length, then the shorter string first: the
// reference's string order (src/scalar_ops.c:78-107)
VG_DEV int str_cmp(const char *a, uint32_t la, const char *b, uint32_t lb) {
    const uint32_t m = la < lb ? la : lb;
    for (uint32_t i = 0; i < m; i++) {
        const unsigned char x = (unsigned char)a[i], y = (unsigned char)b[i];
        if (x != y) return x < y ? -1 : 1;
    }
    return (la > lb) - (la < lb);
}

// fixed-pattern search (src/expr.c:237-268): an empty pattern matches
VG_DEV bool str_contains(const char *s, uint32_t ls, const char *pat, uint32_t lp) {
    if (lp > ls) return false;
    for (uint32_t j = 0; j + lp <= ls; j++) {
        uint32_t k = 0;
        while (k < lp && s[j + k] == pat[k]) k++;
        if (k == lp) return true;
    }
    return false;
}

// double -> int64 toward zero, as C's cast does for values in range; C
// leaves NaN and out-of-range values undefined, here NaN gives 0 and the
// rest saturate
VG_DEV int64_t f2i_trunc(double x) {
    if (x != x) return 0;
    if (x >= 9223372036854775808.0) return INT64_MAX;
    if (x < -9223372036854775808.0) return INT64_MIN;
    return (int64_t)x;
}

VG_DEV int cmp_code(int c, int code) {
    switch (code) {
    case VG_CMP_EQ: return c == 0;
    case VG_CMP_NE: return c != 0;
    case VG_CMP_LT: return c < 0;
    case VG_CMP_LE: return c <= 0;
    case VG_CMP_GT: return c > 0;
    default: return c >= 0;
    }
}

VG_DEV int64_t arith_i64(int64_t a, int64_t b, int op, bool &ok) {
    uint64_t ua = (uint64_t)a, ub = (uint64_t)b;
    switch (op) {
    case '+': return (int64_t)(ua + ub);
    case '-': return (int64_t)(ua - ub);
    case '*': return (int64_t)(ua * ub);
    case '/':
        if (b == 0) { ok = false; return 0; }
        if (b == -1) return (int64_t)(0 - ua);
        return a / b;
    case '%':
        if (b == 0) { ok = false; return 0; }
        if (b == -1) return 0;
        return a % b;
    }
    ok = false;
    return 0;
}

VG_DEV double arith_f64(double a, double b, int op) {
    switch (op) {
    case '+': return __dadd_rn(a, b);
    case '-': return __dsub_rn(a, b);
    case '*': return __dmul_rn(a, b);
    case '/': return __ddiv_rn(a, b);
    default: return fmod(a, b);
    }
}

// Evaluates the program for physical row p.  Returns the top cell.
VG_DEV Cell run_prog(const VgProg &P, const VgCol *cols, int64_t p, uint32_t *err) {
    Cell st[16];
    int sp = 0;
    for (int i = 0; i < P.n; i++) {
        const VgInsn in = P.insn[i];
        switch (in.op) {
        case VI_COL_I64: {
            const VgCol &c = cols[in.a];
            st[sp].ok = vg_valid(c, p);
            st[sp].v = vg_load_bits(c, p);   // bool columns load as 0/1
            sp++;
            break;
        }
        case VI_COL_F64: {
            const VgCol &c = cols[in.a];
            st[sp].ok = vg_valid(c, p);
            uint64_t b = vg_load_bits(c, p);
            if (c.type != VEC_DOUBLE) b = vg_f64_to_bits(vg_i2f((int64_t)b));
            st[sp].v = b;
            sp++;
            break;
        }
        case VI_COL_BOOL: {
            const VgCol &c = cols[in.a];
            st[sp].ok = vg_valid(c, p);
            st[sp].v = vg_load_bits(c, p) ? 1u : 0u;
            sp++;
            break;
        }
        case VI_LIT_I64: case VI_LIT_F64: case VI_LIT_BOOL:
            st[sp].v = (uint64_t)in.imm; st[sp].ok = true; sp++;
            break;
        case VI_LIT_NA:
            st[sp].v = 0; st[sp].ok = false; sp++;
            break;
        case VI_I2F:
            st[sp - 1].v = vg_f64_to_bits(vg_i2f((int64_t)st[sp - 1].v));
            break;
        case VI_ARITH_I64: {
            Cell b = st[--sp], a = st[sp - 1];
            bool ok = a.ok && b.ok;
            int64_t r = ok ? arith_i64((int64_t)a.v, (int64_t)b.v, in.a, ok) : 0;
            st[sp - 1].v = (uint64_t)r; st[sp - 1].ok = ok;
            break;
        }
        case VI_ARITH_F64: {
            Cell b = st[--sp], a = st[sp - 1];
            bool ok = a.ok && b.ok;
            double r = ok ? arith_f64(vg_bits_to_f64(a.v), vg_bits_to_f64(b.v), in.a) : 0.0;
            st[sp - 1].v = vg_f64_to_bits(r); st[sp - 1].ok = ok;
            break;
        }
        case VI_CMP_I64: {
            Cell b = st[--sp], a = st[sp - 1];
            int64_t x = (int64_t)a.v, y = (int64_t)b.v;
            int c = (x > y) - (x < y);
            st[sp - 1].v = (uint64_t)cmp_code(c, in.a); st[sp - 1].ok = a.ok && b.ok;
            break;
        }
        case VI_CMP_F64: {
            Cell b = st[--sp], a = st[sp - 1];
            double x = vg_bits_to_f64(a.v), y = vg_bits_to_f64(b.v);
            int c = (x > y) - (x < y);       // NaN compares as equal
            st[sp - 1].v = (uint64_t)cmp_code(c, in.a); st[sp - 1].ok = a.ok && b.ok;
            break;
        }
        case VI_AND: {   // R's three-valued AND (src/scalar_ops.c:171-175)
            Cell r = st[--sp], l = st[sp - 1];
            Cell o;
            if ((l.ok && !l.v) || (r.ok && !r.v)) { o.ok = true; o.v = 0; }
            else if (l.ok && r.ok) { o.ok = true; o.v = 1; }
            else { o.ok = false; o.v = 0; }
            st[sp - 1] = o;
            break;
        }
        case VI_OR: {    // (src/scalar_ops.c:176-180)
            Cell r = st[--sp], l = st[sp - 1];
            Cell o;
            if ((l.ok && l.v) || (r.ok && r.v)) { o.ok = true; o.v = 1; }
            else if (l.ok && r.ok) { o.ok = true; o.v = 0; }
            else { o.ok = false; o.v = 0; }
            st[sp - 1] = o;
            break;
        }
        case VI_NOT:
            st[sp - 1].v = st[sp - 1].v ? 0u : 1u;
            break;
        case VI_IS_NA:
            st[sp - 1].v = st[sp - 1].ok ? 0u : 1u;
            st[sp - 1].ok = true;
            break;
        case VI_NEG_I64:
            st[sp - 1].v = (uint64_t)(0 - st[sp - 1].v);
            break;
        case VI_NEG_F64:
            st[sp - 1].v ^= 0x8000000000000000ull;
            break;
        case VI_COL_STR: {
            const VgCol &c = cols[in.a];
            const ulonglong2 w = __ldg((const ulonglong2 *)c.data + p);
            st[sp].ok = vg_valid(c, p);
            st[sp].v = w.y;
            st[sp].len = (uint32_t)w.x;
            sp++;
            break;
        }
        case VI_LIT_STR:
            st[sp].v = (uint64_t)(P.pool + in.imm);
            st[sp].len = (uint32_t)in.a;
            st[sp].ok = true;
            sp++;
            break;
        case VI_CMP_STR: {
            Cell b = st[--sp], a = st[sp - 1];
            const bool ok = a.ok && b.ok;
            const int c = ok ? str_cmp((const char *)a.v, a.len, (const char *)b.v, b.len) : 0;
            st[sp - 1].v = (uint64_t)cmp_code(c, in.a); st[sp - 1].ok = ok;
            break;
        }
        case VI_NCHAR:
            st[sp - 1].v = (uint64_t)st[sp - 1].len;
            break;
        case VI_SUBSTR: {   // substr(s, start, stop), 1-based and inclusive (src/expr.c:172-235)
            Cell stop = st[--sp], start = st[--sp];
            Cell &s = st[sp - 1];
            const bool ok = s.ok && start.ok && stop.ok;
            int64_t b0 = (int64_t)((uint64_t)start.v - 1u);
            if (b0 < 0) b0 = 0;
            int64_t e0 = (int64_t)stop.v;
            if (e0 > (int64_t)s.len) e0 = (int64_t)s.len;
            const int64_t n = ok && e0 > b0 ? e0 - b0 : 0;
            s.v = n > 0 ? s.v + (uint64_t)b0 : s.v;
            s.len = (uint32_t)n;
            s.ok = ok;
            break;
        }
        case VI_GREPL:
            st[sp - 1].v = st[sp - 1].ok && str_contains((const char *)st[sp - 1].v, st[sp - 1].len, P.pool + in.imm,
                                                         (uint32_t)in.a) ? 1u : 0u;
            break;
        case VI_F2I:
            st[sp - 1].v = (uint64_t)f2i_trunc(vg_bits_to_f64(st[sp - 1].v));
            break;
        default:
            atomicOr(err, VG_ERR_PROG);
            st[0].ok = false;
            return st[0];
        }
        if (sp < 1 || sp > 15) { atomicOr(err, VG_ERR_PROG); Cell z{0, 0, false}; return z; }
    }
    return st[sp - 1];
}

struct PredArgs {
    VgCol cols[VG_MAX_COLS];
    VgPred pred;
};
struct ProgArgs {
    VgCol cols[VG_MAX_COLS];
    VgProg prog;
};

// Pass 1: keep words (bit j of word w = logical row 32w + j is kept) and
// the number of kept rows per block.
template <bool kUseProg>
__global__ void __launch_bounds__(kThreads)
keep_words_kernel(const PredArgs *pa, const ProgArgs *ga, int64_t n_logical,
                  const int32_t *sel, uint32_t *words, uint32_t *block_counts,
                  uint32_t *err) {
    __shared__ uint32_t warp_cnt[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t block_row0 = (int64_t)blockIdx.x * kRowsPerBlock;
    uint32_t cnt = 0;
    // warp w handles words [w*32, w*32+32) of this block, one per step
    for (int k = 0; k < 32; k++) {
        int64_t wi = (int64_t)blockIdx.x * kThreads + warp * 32 + k;
        int64_t li = wi * 32 + lane;
        bool keep = false;
        if (li < n_logical) {
            int64_t p = sel ? (int64_t)sel[li] : li;
            if (kUseProg) {
                Cell c = run_prog(ga->prog, ga->cols, p, err);
                keep = c.ok && c.v;
            } else {
                keep = pred_keep(pa->pred, pa->cols, p);
            }
        }
        uint32_t m = __ballot_sync(0xFFFFFFFFu, keep);
        if (lane == 0 && wi * 32 < n_logical) words[wi] = m;
        cnt += __popc(m);
    }
    (void)block_row0;
    if (lane == 0) warp_cnt[warp] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int w = 0; w < kThreads / 32; w++) s += warp_cnt[w];
        block_counts[blockIdx.x] = s;
    }
}

// Pass 2: block prefix over earlier blocks, thread prefix inside the block,
// then each thread writes the physical ids of its word's set bits.
__global__ void __launch_bounds__(kThreads)
compact_kernel(int64_t n_logical, const int32_t *sel, const uint32_t *words,
               const uint32_t *block_counts, int n_blocks, int32_t *out,
               int64_t *total) {
    __shared__ uint32_t warp_sum[kThreads / 32];
    __shared__ uint64_t block_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // sum of counts of earlier blocks
    uint64_t acc = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += kThreads) acc += block_counts[b];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, o);
    __shared__ uint64_t part[kThreads / 32];
    if (lane == 0) part[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t s = 0;
        for (int w = 0; w < kThreads / 32; w++) s += part[w];
        block_base = s;
    }
    int64_t wi = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    uint32_t m = (wi * 32 < n_logical) ? words[wi] : 0u;
    uint32_t c = __popc(m);
    // inclusive warp scan
    uint32_t x = c;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    uint32_t wbase = 0;
    for (int w = 0; w < warp; w++) wbase += warp_sum[w];
    uint64_t pos = block_base + wbase + (x - c);
    while (m) {
        int j = __ffs(m) - 1;
        m &= m - 1;
        int64_t li = wi * 32 + j;
        out[pos++] = sel ? sel[li] : (int32_t)li;
    }
    if (blockIdx.x == n_blocks - 1 && threadIdx.x == kThreads - 1) {
        *total = (int64_t)pos;
    }
}

__global__ void eval_kernel(const ProgArgs *ga, int64_t n_logical, const int32_t *sel,
                            int out_type, void *out, uint32_t *out_valid,
                            uint32_t *err) {
    const int lane = threadIdx.x & 31;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // iterate in whole warps so that the validity word is voted at once
    int64_t n_pad = (n_logical + 31) & ~31ll;
    for (int64_t li = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; li < n_pad; li += stride) {
        Cell c{0, 0, false};
        if (li < n_logical) {
            int64_t p = sel ? (int64_t)sel[li] : li;
            c = run_prog(ga->prog, ga->cols, p, err);
            if (out_type == VEC_BOOL) ((uint8_t *)out)[li] = (uint8_t)(c.ok ? (c.v ? 1 : 0) : 0);
            else if (out_type == VEC_STRING) ((VgStrView *)out)[li] = vg_str_view((const char *)c.v, c.ok ? c.len : 0u);
            else ((uint64_t *)out)[li] = c.ok ? c.v : 0;
        }
        uint32_t m = __ballot_sync(0xFFFFFFFFu, c.ok && li < n_logical);
        if (lane == 0) out_valid[li >> 5] = m;
    }
}

__global__ void gather_kernel(VgCol c, const int32_t *idx, int64_t n_out, int null_if_neg,
                              void *out, uint32_t *out_valid) {
    const int lane = threadIdx.x & 31;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t n_pad = (n_out + 31) & ~31ll;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n_pad; j += stride) {
        bool ok = false;
        if (j < n_out) {
            int64_t p = idx ? (int64_t)idx[j] : j;
            if (p >= 0) {
                ok = vg_valid(c, p);
                if (c.type == VEC_BOOL) ((uint8_t *)out)[j] = ok ? __ldg((const uint8_t *)c.data + p) : 0;
                else if (c.type == VEC_STRING)
                    ((ulonglong2 *)out)[j] = ok ? __ldg((const ulonglong2 *)c.data + p) : make_ulonglong2(0, 0);
                else ((uint64_t *)out)[j] = ok ? vg_load_bits(c, p) : 0;
            } else {
                if (c.type == VEC_BOOL) ((uint8_t *)out)[j] = 0;
                else if (c.type == VEC_STRING) ((ulonglong2 *)out)[j] = make_ulonglong2(0, 0);
                else ((uint64_t *)out)[j] = 0;
            }
        }
        (void)null_if_neg;
        uint32_t m = __ballot_sync(0xFFFFFFFFu, ok);
        if (lane == 0) out_valid[j >> 5] = m;
    }
}

__global__ void gather_into_kernel(VgCol c, const int32_t *idx, int64_t n, void *out,
                                   uint32_t *out_valid, int64_t row0) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        int64_t p = idx ? (int64_t)idx[j] : j;
        bool ok = vg_valid(c, p);
        int64_t d = row0 + j;
        if (c.type == VEC_BOOL) ((uint8_t *)out)[d] = ok ? __ldg((const uint8_t *)c.data + p) : 0;
        else if (c.type == VEC_STRING)
            ((ulonglong2 *)out)[d] = ok ? __ldg((const ulonglong2 *)c.data + p) : make_ulonglong2(0, 0);
        else ((uint64_t *)out)[d] = ok ? vg_load_bits(c, p) : 0;
        if (ok) atomicOr(out_valid + (d >> 5), 1u << (d & 31));
    }
}

char g_err_msg[256];

int check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        snprintf(g_err_msg, sizeof(g_err_msg), "%s: %s", what, cudaGetErrorString(e));
        return -1;
    }
    return 0;
}

int grid_for(int64_t n, int threads) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    int64_t want = (n + threads - 1) / threads;
    int64_t cap = (int64_t)sms * 16;
    if (want > cap) want = cap;
    if (want < 1) want = 1;
    return (int)want;
}

// scratch layout: [args struct][keep words][block counts][total]
struct FilterScratch {
    void *args; uint32_t *words; uint32_t *counts; int64_t *total; uint32_t *err;
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

bool carve(void *base, size_t bytes, int64_t n_logical, size_t args_bytes, FilterScratch &fs) {
    int64_t n_blocks = (n_logical + kRowsPerBlock - 1) / kRowsPerBlock;
    if (n_blocks < 1) n_blocks = 1;
    size_t off = 0;
    char *p = (char *)base;
    fs.args = p + off; off += align256(args_bytes);
    fs.words = (uint32_t *)(p + off); off += align256((size_t)n_blocks * kThreads * 4);
    fs.counts = (uint32_t *)(p + off); off += align256((size_t)n_blocks * 4);
    fs.total = (int64_t *)(p + off); off += 256;
    fs.err = (uint32_t *)(p + off); off += 256;
    return off <= bytes;
}


// min, max and number of the valid values of an int64 column:
// out[0] = min, out[1] = max, out[2] = count (out preset by minmax_init_kernel)
__global__ void minmax_init_kernel(long long *out) {
    out[0] = 0x7FFFFFFFFFFFFFFFll;
    out[1] = (long long)0x8000000000000000ull;
    out[2] = 0;
}

// Each thread takes kMinmaxU rows per step (blockDim apart: coalesced) and
// issues their loads before it uses them, so that enough bytes are in
// flight to keep HBM busy.
constexpr int kMinmaxU = 4;

__global__ void minmax_i64_kernel(VgCol c, int64_t n, long long *out) {
    long long lo = 0x7FFFFFFFFFFFFFFFll, hi = (long long)0x8000000000000000ull, cnt = 0;
    const long long *v = (const long long *)c.data;
    const int64_t step = (int64_t)gridDim.x * blockDim.x * kMinmaxU;
    for (int64_t r0 = (int64_t)blockIdx.x * blockDim.x * kMinmaxU + threadIdx.x; r0 < n; r0 += step) {
        long long x[kMinmaxU];
        uint32_t w[kMinmaxU];
#pragma unroll
        for (int u = 0; u < kMinmaxU; u++) {
            const int64_t r = r0 + (int64_t)u * blockDim.x;
            x[u] = 0;
            w[u] = 0;
            if (r < n) {
                x[u] = __ldg(v + r);
                w[u] = c.valid ? __ldg(c.valid + ((r + c.voff) >> 5)) : 0xFFFFFFFFu;
            }
        }
#pragma unroll
        for (int u = 0; u < kMinmaxU; u++) {
            const int64_t r = r0 + (int64_t)u * blockDim.x;
            if (r >= n || !((w[u] >> ((r + c.voff) & 31)) & 1u)) continue;
            lo = x[u] < lo ? x[u] : lo;
            hi = x[u] > hi ? x[u] : hi;
            cnt++;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        long long l2 = __shfl_xor_sync(0xFFFFFFFFu, lo, o);
        long long h2 = __shfl_xor_sync(0xFFFFFFFFu, hi, o);
        cnt += __shfl_xor_sync(0xFFFFFFFFu, cnt, o);
        lo = l2 < lo ? l2 : lo;
        hi = h2 > hi ? h2 : hi;
    }
    // one combine per block: the three result words are single addresses
    __shared__ long long s_lo, s_hi;
    __shared__ unsigned long long s_cnt;
    if (threadIdx.x == 0) {
        s_lo = 0x7FFFFFFFFFFFFFFFll;
        s_hi = (long long)0x8000000000000000ull;
        s_cnt = 0;
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0 && cnt > 0) {
        atomicMin(&s_lo, lo);
        atomicMax(&s_hi, hi);
        atomicAdd(&s_cnt, (unsigned long long)cnt);
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_cnt > 0) {
        atomicMin(out + 0, s_lo);
        atomicMax(out + 1, s_hi);
        atomicAdd((unsigned long long *)out + 2, s_cnt);
    }
}

// Pass 1 for general programs, whose rows cost far more than a range
// test: one warp per keep word (32 rows), so that a batch of any size
// spreads over every SM; each word's count is added to its 256-word
// block's count (zeroed before the launch), the layout pass 2 reads.
__global__ void __launch_bounds__(kThreads)
keep_words_prog_kernel(const ProgArgs *ga, int64_t n_logical, const int32_t *sel, uint32_t *words,
                       uint32_t *block_counts, uint32_t *err) {
    const int lane = threadIdx.x & 31;
    const int64_t wi = ((int64_t)blockIdx.x * kThreads + threadIdx.x) >> 5;
    const int64_t li = wi * 32 + lane;
    bool keep = false;
    if (li < n_logical) {
        const int64_t p = sel ? (int64_t)sel[li] : li;
        const Cell c = run_prog(ga->prog, ga->cols, p, err);
        keep = c.ok && c.v;
    }
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, keep);
    if (lane == 0 && wi * 32 < n_logical) {
        words[wi] = m;
        if (m) atomicAdd(block_counts + wi / kThreads, (uint32_t)__popc(m));
    }
}

template <bool kUseProg>
int run_filter(const void *args, size_t args_bytes, int64_t n_logical, const int32_t *d_sel_in,
               int32_t *d_sel_out, int64_t *h_count, void *d_scratch, size_t scratch_bytes,
               cudaStream_t s) {
    FilterScratch fs;
    if (!carve(d_scratch, scratch_bytes, n_logical, args_bytes, fs)) {
        snprintf(g_err_msg, sizeof(g_err_msg), "filter scratch too small");
        return -1;
    }
    if (n_logical <= 0) { *h_count = 0; return 0; }
    int n_blocks = (int)((n_logical + kRowsPerBlock - 1) / kRowsPerBlock);
    if (check(cudaMemcpyAsync(fs.args, args, args_bytes, cudaMemcpyHostToDevice, s), "filter args")) return -1;
    if (check(cudaMemsetAsync(fs.err, 0, 4, s), "filter err")) return -1;
    vg_prof_begin(VG_PROF_FILTER, s);
    if (kUseProg) {
        const int64_t n_words = (n_logical + 31) / 32;
        if (check(cudaMemsetAsync(fs.counts, 0, (size_t)n_blocks * 4, s), "filter counts")) return -1;
        { keep_words_prog_kernel<<<(unsigned)((n_words + kThreads / 32 - 1) / (kThreads / 32)), kThreads, 0, s>>>(
            (const ProgArgs *)fs.args, n_logical, d_sel_in, fs.words, fs.counts, fs.err); vg_launch_counter++; }
    } else {
        keep_words_kernel<false><<<n_blocks, kThreads, 0, s>>>(
            (const PredArgs *)fs.args, (const ProgArgs *)fs.args, n_logical, d_sel_in,
            fs.words, fs.counts, fs.err);
        vg_launch_counter++;
    }
    { compact_kernel<<<n_blocks, kThreads, 0, s>>>(n_logical, d_sel_in, fs.words, fs.counts,
                                                 n_blocks, d_sel_out, fs.total); vg_launch_counter++; }
    vg_prof_end(VG_PROF_FILTER, s);
    int64_t tot = 0;
    uint32_t err = 0;
    if (check(cudaMemcpyAsync(&tot, fs.total, 8, cudaMemcpyDeviceToHost, s), "filter count")) return -1;
    if (check(cudaMemcpyAsync(&err, fs.err, 4, cudaMemcpyDeviceToHost, s), "filter err")) return -1;
    if (check(cudaStreamSynchronize(s), "filter")) return -1;
    if (err) { snprintf(g_err_msg, sizeof(g_err_msg), "filter: invalid expression program"); return -1; }
    *h_count = tot;
    return 0;
}

}  // namespace

extern "C" {

const char *vgk_last_cuda_error(void) { return g_err_msg; }

int vgk_num_sms(void) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

size_t vgk_filter_scratch_bytes(int64_t n_logical) {
    int64_t n_blocks = (n_logical + kRowsPerBlock - 1) / kRowsPerBlock;
    if (n_blocks < 1) n_blocks = 1;
    size_t a = sizeof(PredArgs) > sizeof(ProgArgs) ? sizeof(PredArgs) : sizeof(ProgArgs);
    return align256(a) + align256((size_t)n_blocks * kThreads * 4) +
           align256((size_t)n_blocks * 4) + 512;
}

int vgk_filter_pred(const VgCol *cols, int n_cols, const VgPred *pred, int64_t n_rows,
                    const int32_t *d_sel_in, int64_t sel_n, int32_t *d_sel_out,
                    int64_t *h_count, void *d_scratch, size_t scratch_bytes, vg_stream_t s) {
    PredArgs a;
    memset(&a, 0, sizeof(a));
    if (n_cols > VG_MAX_COLS) { snprintf(g_err_msg, sizeof(g_err_msg), "too many columns"); return -1; }
    for (int i = 0; i < n_cols; i++) a.cols[i] = cols[i];
    a.pred = *pred;
    int64_t n_logical = d_sel_in ? sel_n : n_rows;
    return run_filter<false>(&a, sizeof(a), n_logical, d_sel_in, d_sel_out, h_count, d_scratch,
                             scratch_bytes, (cudaStream_t)s);
}

int vgk_filter_prog(const VgCol *cols, int n_cols, const VgProg *prog, int64_t n_rows,
                    const int32_t *d_sel_in, int64_t sel_n, int32_t *d_sel_out,
                    int64_t *h_count, void *d_scratch, size_t scratch_bytes, vg_stream_t s) {
    ProgArgs a;
    memset(&a, 0, sizeof(a));
    if (n_cols > VG_MAX_COLS) { snprintf(g_err_msg, sizeof(g_err_msg), "too many columns"); return -1; }
    for (int i = 0; i < n_cols; i++) a.cols[i] = cols[i];
    a.prog = *prog;
    int64_t n_logical = d_sel_in ? sel_n : n_rows;
    return run_filter<true>(&a, sizeof(a), n_logical, d_sel_in, d_sel_out, h_count, d_scratch,
                            scratch_bytes, (cudaStream_t)s);
}

int vgk_eval_prog(const VgCol *cols, int n_cols, const VgProg *prog, int64_t n_rows,
                  const int32_t *d_sel, int64_t sel_n, void *d_out, uint32_t *d_out_valid,
                  vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    int64_t n_logical = d_sel ? sel_n : n_rows;
    if (n_logical <= 0) return 0;
    ProgArgs a;
    memset(&a, 0, sizeof(a));
    if (n_cols > VG_MAX_COLS) { snprintf(g_err_msg, sizeof(g_err_msg), "too many columns"); return -1; }
    for (int i = 0; i < n_cols; i++) a.cols[i] = cols[i];
    a.prog = *prog;
    void *dargs = nullptr;
    if (check(cudaMallocAsync(&dargs, align256(sizeof(a)) + 256, st), "eval args")) return -1;
    uint32_t *derr = (uint32_t *)((char *)dargs + align256(sizeof(a)));
    cudaMemcpyAsync(dargs, &a, sizeof(a), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(derr, 0, 4, st);
    { eval_kernel<<<grid_for(n_logical, 256), 256, 0, st>>>((const ProgArgs *)dargs, n_logical, d_sel,
                                                           prog->result_type, d_out, d_out_valid, derr); vg_launch_counter++; }
    uint32_t err = 0;
    cudaMemcpyAsync(&err, derr, 4, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(dargs, st);
    if (check(cudaStreamSynchronize(st), "eval")) return -1;
    if (err) { snprintf(g_err_msg, sizeof(g_err_msg), "eval: invalid expression program"); return -1; }
    return 0;
}

int vgk_gather(const VgCol *col, const int32_t *d_idx, int64_t n_out, int null_if_negative,
               void *d_out, uint32_t *d_out_valid, vg_stream_t s) {
    if (n_out <= 0) return 0;
    cudaStream_t st = (cudaStream_t)s;
    { gather_kernel<<<grid_for(n_out, 256), 256, 0, st>>>(*col, d_idx, n_out, null_if_negative,
                                                         d_out, d_out_valid); vg_launch_counter++; }
    return check(cudaGetLastError(), "gather");
}

int vgk_gather_into(const VgCol *col, const int32_t *d_idx, int64_t n, void *d_out,
                    uint32_t *d_out_valid, int64_t row0, vg_stream_t s) {
    if (n <= 0) return 0;
    cudaStream_t st = (cudaStream_t)s;
    { gather_into_kernel<<<grid_for(n, 256), 256, 0, st>>>(*col, d_idx, n, d_out, d_out_valid, row0); vg_launch_counter++; }
    return check(cudaGetLastError(), "gather into");
}

int vgk_col_minmax_i64(const VgCol *col, int64_t n, int64_t *d_out, int64_t *h_out, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    { minmax_init_kernel<<<1, 1, 0, st>>>((long long *)d_out); vg_launch_counter++; }
    if (n > 0) {
        minmax_i64_kernel<<<grid_for((n + kMinmaxU - 1) / kMinmaxU, 256), 256, 0, st>>>(*col, n, (long long *)d_out);
        vg_launch_counter++;
    }
    if (check(cudaMemcpyAsync(h_out, d_out, 24, cudaMemcpyDeviceToHost, st), "column min/max")) return -1;
    return check(cudaStreamSynchronize(st), "column min/max");
}

}  // extern "C"
