// k_hashjoin.cu -- hash-join build and probe on sm_103a.
//
// Replaces the reference's JoinHT (src/join.c:23-150), join_build
// (src/join.c:156-220) and join_probe_one (src/join.c:262-480):
//  * build: one device pass inserts every non-NA build key into an
//    open-addressing table with one slot per distinct key and counts rows
//    per key.  Single-key tables claim 16-byte {key, start, count} slots
//    with one 64-bit CAS on the key (no locks, no fences; one sector per
//    probe); composite keys use per-slot locks.  If any key repeats, a
//    stable radix sort of (slot, build row) lays each key's rows out in
//    ascending row order, so the probe can emit them in the reference's
//    descending order (its chains are built by head insertion,
//    src/join.c:55-56);
//  * probe: count -> exclusive scan -> emit (probe row, build row) pairs in
//    the reference's output order: probe rows in order, matches in
//    descending build row, then (LEFT/FULL) the unmatched probe rows of the
//    batch (src/join.c:438-450).  SEMI/ANTI emit a selection vector.

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "k_common.cuh"

extern "C" {
size_t vgk_sort_pairs_scratch(int64_t n);
int vgk_sort_pairs(uint64_t *keys, int32_t *vals, int64_t n, int key_bits, void *scratch,
                   size_t scratch_bytes, vg_stream_t s);
const char *vgk_sort_last_error(void);
size_t vgk_scan_scratch(int64_t n);
int vgk_exclusive_scan(const int32_t *in, int64_t n, int64_t *out, int64_t *d_total, void *scratch,
                       size_t scratch_bytes, vg_stream_t s);
}

namespace {

char g_err[256];
int check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof(g_err), "%s: %s", what, cudaGetErrorString(e));
        return -1;
    }
    return 0;
}
size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

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

struct KeyArgs {
    int n_keys;
    int32_t conv[VG_MAX_KEYS];
    int32_t types[VG_MAX_KEYS];
    VgCol cols[VG_MAX_KEYS];
};

// normalised key words of row r; false if any key is NA or NaN (never matches)
VG_DEV bool key_words(const KeyArgs &K, int64_t r, uint64_t *k) {
#pragma unroll
    for (int i = 0; i < VG_MAX_KEYS; i++) {
        if (i >= K.n_keys) break;
        const VgCol &c = K.cols[i];
        if (!vg_valid(c, r)) return false;
        uint64_t b = vg_load_bits(c, r);
        if (K.conv[i]) b = vg_f64_to_bits(vg_i2f((int64_t)b));
        if (K.types[i] == VEC_DOUBLE && vg_is_nan_bits(b)) return false;
        k[i] = vg_norm_key(b, K.types[i]);
    }
    return true;
}

VG_DEV int32_t *jt_start_ptr(const VgJoinTable &jt, int64_t slot) {
    return jt.slots ? &jt.slots[slot].start : jt.start + slot;
}
VG_DEV int32_t *jt_count_ptr(const VgJoinTable &jt, int64_t slot) {
    return jt.slots ? &jt.slots[slot].count : jt.count + slot;
}

// Payload columns written by the build itself (direct tables).
struct PayArgs {
    VgCol c0, c1;
    int n_cols;
    VgJPay *pay;             // NULL: none requested
    int narrow;              // the column a VgJPay16 entry narrows (int64 / bool), -1: none
    ulonglong2 *payrow;      // pass 1: each build row's would-be compact entry, in row order (or NULL)
};

// Whether the payload fits VgJPay16 entries (decided from the statistics of
// pass 1, the same way on the device and on the host): one column, or two of which `narrow` is a bool
// column or an int64 column whose valid values span less than 2^32 (none
// valid: stored as 0).  *mn: the narrowed column's minimum.
__host__ __device__ inline bool pay16_fits(int n_cols, int narrow, int narrow_type, const long long *mm,
                                           long long *mn) {
    *mn = 0;
    if (n_cols == 1) return true;
    if (n_cols != 2 || narrow < 0) return false;
    if (narrow_type == VEC_BOOL) return true;
    if (narrow_type != VEC_INT64) return false;
    if (mm[3 * narrow + 2] == 0) return true;
    if ((unsigned long long)mm[3 * narrow + 1] - (unsigned long long)mm[3 * narrow] > 0xFFFFFFFFull) return false;
    *mn = mm[3 * narrow];
    return true;
}

// Empties the table (init_slots) and / or zeroes the payload copy; resets
// the counters and the payload min / max words.
__global__ void jt_init_kernel(VgJoinTable jt, uint32_t *counters, VgJPay *pay, int init_slots, long long *mm) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n = jt.slots ? jt.cap + 1 : jt.cap;
    if (mm && blockIdx.x == 0 && threadIdx.x < 2) {
        mm[3 * threadIdx.x + 0] = 0x7FFFFFFFFFFFFFFFll;
        mm[3 * threadIdx.x + 1] = (long long)0x8000000000000000ull;
        mm[3 * threadIdx.x + 2] = 0;
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n && (pay || init_slots); i += stride) {
        if (pay) {
            ulonglong2 *o = (ulonglong2 *)(pay + i);
            o[0] = make_ulonglong2(0ull, 0ull);
            o[1] = make_ulonglong2(0ull, 0ull);
        }
        if (!init_slots) continue;
        if (jt.slots) {
            jt.slots[i].key = VG_JEMPTY;
            jt.slots[i].start = 0;
            jt.slots[i].count = 0;
        } else {
            jt.state[i] = 0;
            jt.count[i] = 0;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < 8) counters[threadIdx.x] = 0;
}

// single key: claim a slot with one CAS on its key word (direct tables:
// the key's own slot; the host sized the range from the build keys)
VG_DEV int64_t insert_single(const VgJoinTable &jt, uint64_t k, uint32_t *counters) {
    if (jt.direct) {
        const int64_t d = jt_direct_slot(jt, k);
        if (d < 0) { atomicOr(counters + 2, VG_ERR_FULL); return -1; }
        jt.slots[d].key = k;                // every writer stores the same word
        return d;
    }
    if (k == VG_JEMPTY) return jt.cap;      // the marker value has its own slot
    const int64_t mask = jt.cap - 1;
    int64_t slot = (int64_t)(vg_jhash(&k, 1) & (uint64_t)mask);
    for (int64_t probe = 0; probe < jt.cap; probe++) {
        unsigned long long *kp = (unsigned long long *)&jt.slots[slot].key;
        unsigned long long cur = *(volatile unsigned long long *)kp;
        if (cur == k) return slot;
        if (cur == VG_JEMPTY) {
            unsigned long long prev = atomicCAS(kp, VG_JEMPTY, k);
            if (prev == VG_JEMPTY || prev == k) return slot;
        }
        slot = (slot + 1) & mask;
    }
    atomicOr(counters + 2, VG_ERR_FULL);
    return -1;
}

// composite keys: per-slot lock (0 empty, 1 being written, 2 ready)
VG_DEV int64_t insert_multi(const VgJoinTable &jt, const uint64_t *k, int nk, uint32_t *counters) {
    const int64_t mask = jt.cap - 1;
    int64_t slot = (int64_t)(vg_jhash(k, nk) & (uint64_t)mask);
    for (int64_t probe = 0; probe < jt.cap; probe++) {
        // acquire loads of the state order the key reads after state 2
        uint32_t st = vg_ld_acquire(jt.state + slot);
        if (st == 0) {
            uint32_t prev = atomicCAS(jt.state + slot, 0u, 1u);
            if (prev == 0u) {
                for (int i = 0; i < nk; i++) jt.keys[(int64_t)i * jt.cap + slot] = k[i];
                __threadfence();
                atomicExch(jt.state + slot, 2u);
                return slot;
            }
            st = vg_ld_acquire(jt.state + slot);
        }
        int spins = 0;
        while (st == 1u) {
            if (++spins > VG_SPIN_LIMIT) { atomicOr(counters + 2, VG_ERR_WAIT); return -1; }
            __nanosleep(32);
            st = vg_ld_acquire(jt.state + slot);
        }
        bool eq = true;
        for (int i = 0; i < nk && eq; i++)
            eq = *(volatile uint64_t *)(jt.keys + (int64_t)i * jt.cap + slot) == k[i];
        if (eq) return slot;
        slot = (slot + 1) & mask;
    }
    atomicOr(counters + 2, VG_ERR_FULL);
    return -1;
}

// counters: [0] distinct keys, [1] max rows per key, [2] error bits.
// Every warp runs the same number of iterations (the row index is the
// block's base plus the lane), so the per-warp counter updates can be
// combined with full-warp votes: one atomic per warp instead of one per row.
__global__ void jt_insert_kernel(VgJoinTable jt, KeyArgs K, int64_t n, int32_t *rslot,
                                 uint32_t *counters) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x; b < n; b += stride) {
        const int64_t r = b + threadIdx.x;
        bool first = false;
        uint32_t dup = 0;
        if (r < n) {
            uint64_t k[VG_MAX_KEYS];
            int64_t found = -1;
            if (key_words(K, r, k))
                found = jt.slots ? insert_single(jt, k[0], counters) : insert_multi(jt, k, K.n_keys, counters);
            if (found >= 0) {
                int32_t old = atomicAdd(jt_count_ptr(jt, found), 1);
                if (old == 0) {
                    first = true;
                    *jt_start_ptr(jt, found) = (int32_t)r;   // final when keys are unique
                } else {
                    dup = (uint32_t)(old + 1);
                }
            }
            rslot[r] = (int32_t)found;
        }
        const unsigned nfirst = __popc(__ballot_sync(0xFFFFFFFFu, first));
        const unsigned mx = __reduce_max_sync(0xFFFFFFFFu, dup);
        if (lane == 0) {
            if (nfirst) atomicAdd(counters + 0, nfirst);
            if (mx) atomicMax(counters + 1, mx);
        }
    }
}

// Payload copy of the slot table: per slot the key, the build row and the
// values and validity of up to two build columns of that row.
__global__ void jt_pay_kernel(VgJoinTable jt, VgCol c0, VgCol c1, int n_cols, VgJPay *pay) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s <= jt.cap; s += stride) {
        const VgJSlot e = jt_slot(jt.slots + s);
        uint64_t p0 = 0, p1 = 0;
        uint32_t meta = 0;
        if (e.count > 0 && (jt.direct || s == jt.cap || e.key != VG_JEMPTY)) {
            const int64_t r = e.start;
            meta = 1u;
            if (n_cols > 0) {
                p0 = vg_load_bits(c0, r);
                if (vg_valid(c0, r)) meta |= 2u;
            }
            if (n_cols > 1) {
                p1 = vg_load_bits(c1, r);
                if (vg_valid(c1, r)) meta |= 4u;
            }
        }
        ulonglong2 *o = (ulonglong2 *)(pay + s);
        o[0] = make_ulonglong2(e.key, (unsigned long long)(uint32_t)e.start | ((unsigned long long)meta << 32));
        o[1] = make_ulonglong2(p0, p1);
    }
}

// Direct tables: every build row writes its key's own slot; the counts are
// non-returning adds, and the distinct / duplicate counters come from a
// pass over the slots afterwards (jt_count_kernel).  With duplicates the
// start written here is replaced by the sorted layout (seg_start_kernel).
__global__ void jt_insert_direct_kernel(VgJoinTable jt, KeyArgs K, int64_t n, int32_t *rslot,
                                        uint32_t *counters, PayArgs P) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    uint64_t k[VG_MAX_KEYS];
    int64_t d = -1;
    if (key_words(K, r, k)) {
        d = jt_direct_slot(jt, k[0]);
        if (d < 0) {
            atomicOr(counters + 2, VG_ERR_FULL);
        } else {
            jt.slots[d].key = k[0];
            jt.slots[d].start = (int32_t)r;
            atomicAdd(&jt.slots[d].count, 1);
            if (P.pay) {
                // the payload entry of this key (meaningful when keys are unique)
                uint64_t p0 = 0, p1 = 0;
                uint32_t meta = 1u;
                if (P.n_cols > 0) {
                    p0 = vg_load_bits(P.c0, r);
                    if (vg_valid(P.c0, r)) meta |= 2u;
                }
                if (P.n_cols > 1) {
                    p1 = vg_load_bits(P.c1, r);
                    if (vg_valid(P.c1, r)) meta |= 4u;
                }
                vg_st256(P.pay + d, k[0], (unsigned long long)(uint32_t)r | ((unsigned long long)meta << 32), p0,
                         p1);
            }
        }
    }
    rslot[r] = (int32_t)d;
}

// Direct tables with a payload copy, built without random writes to the
// large tables.  Pass 1: every build row records itself in rowof[key - min]
// (4 bytes per key: small enough to stay in L2) with the validity bits of
// its two payload values in bits 29 and 30, counts the rows it recorded, and
// reports min, max and count of the valid values of int64 payload columns
// (mm, 3 words per column); for a payload that may take compact entries it
// also writes each row's would-be entry in row order.  Pass 2 counts the
// slots some row holds (fewer than rows recorded: a key repeats) and, if
// the payload fits compact entries, gathers them by slot (coalesced writes,
// jt_pay16_gather_kernel).  Otherwise, once the host has read the counts,
// each recorded row writes its key's full entry (reading its payload values
// in row order) and the entries of keys no row has are cleared last.
//
// Each thread takes kBuildU rows per step (blockDim apart, so every load
// stays coalesced) and issues all their loads before it uses any: a row's
// work is a short chain of dependent loads, and one row per step leaves too
// few bytes in flight to keep HBM busy.  The step loop runs on the block's
// first row so that every thread of a warp takes the same number of steps.
// A direct table has a single key (node_join.c builds one only then).
constexpr int32_t kRowBits = 29;                       // build rows < 2^29
constexpr uint32_t kRowMask = (1u << kRowBits) - 1u;
constexpr int kBuildU = 4;
static_assert(sizeof(VgJPay) == 32, "one 32-byte store per payload entry");

// validity word of row r (all ones for a column without a bitmap), and the
// bit of row r in it
VG_DEV uint32_t valid_word(const VgCol &c, int64_t r) {
    return c.valid ? __ldg(c.valid + ((r + c.voff) >> 5)) : 0xFFFFFFFFu;
}
VG_DEV bool valid_bit(const VgCol &c, int64_t r, uint32_t w) { return (w >> ((r + c.voff) & 31)) & 1u; }

// key_words for a single key from its preloaded bits and validity word
VG_DEV bool key_word_from(const KeyArgs &K, int64_t r, uint64_t b, uint32_t vw, uint64_t *k) {
    if (!valid_bit(K.cols[0], r, vw)) return false;
    if (K.conv[0]) b = vg_f64_to_bits(vg_i2f((int64_t)b));
    if (K.types[0] == VEC_DOUBLE && vg_is_nan_bits(b)) return false;
    k[0] = vg_norm_key(b, K.types[0]);
    return true;
}

__global__ void jt_rows_direct_kernel(VgJoinTable jt, KeyArgs K, int64_t n, int32_t *rslot, uint32_t *counters,
                                      PayArgs P, uint32_t *rowof, long long *mm) {
    // per-thread min / max / count, then one combine per block (the
    // statistic words are single addresses)
    long long lo[2] = {0x7FFFFFFFFFFFFFFFll, 0x7FFFFFFFFFFFFFFFll};
    long long hi[2] = {(long long)0x8000000000000000ull, (long long)0x8000000000000000ull};
    unsigned long long cnt[2] = {0, 0};
    unsigned long long recorded = 0;
    const int64_t step = (int64_t)gridDim.x * blockDim.x * kBuildU;
    for (int64_t b0 = (int64_t)blockIdx.x * blockDim.x * kBuildU; b0 < n; b0 += step) {
        uint64_t kb[kBuildU], pb[2][kBuildU];
        uint32_t kv[kBuildU], pv[2][kBuildU];
#pragma unroll
        for (int u = 0; u < kBuildU; u++) {
            const int64_t r = b0 + (int64_t)u * blockDim.x + threadIdx.x;
            kb[u] = 0;
            kv[u] = 0;
            pb[0][u] = pb[1][u] = 0;
            pv[0][u] = pv[1][u] = 0;
            if (r < n) {
                kb[u] = vg_load_bits(K.cols[0], r);
                kv[u] = valid_word(K.cols[0], r);
#pragma unroll
                for (int c = 0; c < 2; c++) {
                    if (c >= P.n_cols) continue;
                    const VgCol &col = c == 0 ? P.c0 : P.c1;
                    pv[c][u] = valid_word(col, r);
                    if (col.type == VEC_INT64 || P.payrow) pb[c][u] = vg_load_bits(col, r);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kBuildU; u++) {
            const int64_t r = b0 + (int64_t)u * blockDim.x + threadIdx.x;
            if (r >= n) break;
            uint64_t k[VG_MAX_KEYS];
            int64_t d = -1;
            if (key_word_from(K, r, kb[u], kv[u], k)) {
                d = jt_direct_slot(jt, k[0]);
                if (d < 0) atomicOr(counters + 2, VG_ERR_FULL);
            }
            uint32_t vb = 0;                           // validity of the payload values
            if (P.n_cols > 0 && valid_bit(P.c0, r, pv[0][u])) vb |= 1u;
            if (P.n_cols > 1 && valid_bit(P.c1, r, pv[1][u])) vb |= 2u;
            // rows with a key in range record themselves (counted: fewer
            // keys present than rows recorded means a key repeats)
            if (d >= 0) {
                rowof[d] = (uint32_t)r | (vb << kRowBits);
                recorded++;
            }
            rslot[r] = (int32_t)d;
            if (P.payrow) {
                // the kept column whole, the narrowed one's low 32 bits (its
                // minimum is known only at the end of this pass)
                const uint64_t a = P.n_cols == 1 ? pb[0][u] : (P.narrow == 0 ? pb[1][u] : pb[0][u]);
                const uint64_t nv = P.narrow == 0 ? pb[0][u] : pb[1][u];
                P.payrow[r] = make_ulonglong2(a, P.n_cols == 1 ? 0ull : (unsigned long long)(uint32_t)nv);
            }
#pragma unroll
            for (int c = 0; c < 2; c++) {
                if (c >= P.n_cols || !((vb >> c) & 1u)) continue;
                const VgCol &col = c == 0 ? P.c0 : P.c1;
                if (col.type != VEC_INT64) continue;
                const long long x = (long long)pb[c][u];
                lo[c] = x < lo[c] ? x : lo[c];
                hi[c] = x > hi[c] ? x : hi[c];
                cnt[c]++;
            }
        }
    }
    __shared__ long long s_lo[2], s_hi[2];
    __shared__ unsigned long long s_cnt[2];
    if (threadIdx.x < 2) {
        s_lo[threadIdx.x] = 0x7FFFFFFFFFFFFFFFll;
        s_hi[threadIdx.x] = (long long)0x8000000000000000ull;
        s_cnt[threadIdx.x] = 0;
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < 2; c++) {
        for (int o = 16; o > 0; o >>= 1) {
            const long long l2 = __shfl_xor_sync(0xFFFFFFFFu, lo[c], o);
            const long long h2 = __shfl_xor_sync(0xFFFFFFFFu, hi[c], o);
            cnt[c] += __shfl_xor_sync(0xFFFFFFFFu, cnt[c], o);
            lo[c] = l2 < lo[c] ? l2 : lo[c];
            hi[c] = h2 > hi[c] ? h2 : hi[c];
        }
        if ((threadIdx.x & 31) == 0 && cnt[c]) {
            atomicMin(s_lo + c, lo[c]);
            atomicMax(s_hi + c, hi[c]);
            atomicAdd(s_cnt + c, cnt[c]);
        }
    }
    for (int o = 16; o > 0; o >>= 1) recorded += __shfl_xor_sync(0xFFFFFFFFu, recorded, o);
    if ((threadIdx.x & 31) == 0 && recorded) atomicAdd((unsigned long long *)(counters + 4), recorded);
    __syncthreads();
    if (threadIdx.x < 2 && threadIdx.x < P.n_cols && s_cnt[threadIdx.x]) {
        const int c = threadIdx.x;
        atomicMin(mm + 3 * c, s_lo[c]);
        atomicMax(mm + 3 * c + 1, s_hi[c]);
        atomicAdd((unsigned long long *)mm + 3 * c + 2, s_cnt[c]);
    }
}

// Pass 2 (as verify + gather in one): each row that its key's entry names
// writes the entry (one 32-byte store; the payload copy is 32-byte aligned),
// its payload values read where they are (coalesced); a row whose key names
// another row reports a repeated key.  Entries of keys no row has are
// written by jt_pay_absent_kernel.
__global__ void jt_pay_scatter_kernel(VgJoinTable jt, const uint32_t *rowof, const int32_t *rslot, int64_t n,
                                      PayArgs P, uint32_t *counters) {
    const int64_t step = (int64_t)gridDim.x * blockDim.x * kBuildU;
    for (int64_t b0 = (int64_t)blockIdx.x * blockDim.x * kBuildU; b0 < n; b0 += step) {
        int32_t d[kBuildU];
        uint64_t p0[kBuildU], p1[kBuildU];
#pragma unroll
        for (int u = 0; u < kBuildU; u++) {
            const int64_t r = b0 + (int64_t)u * blockDim.x + threadIdx.x;
            d[u] = -1;
            p0[u] = p1[u] = 0;
            if (r < n) {
                d[u] = rslot[r];
                if (P.n_cols > 0) p0[u] = vg_load_bits(P.c0, r);
                if (P.n_cols > 1) p1[u] = vg_load_bits(P.c1, r);
            }
        }
        uint32_t v[kBuildU];
#pragma unroll
        for (int u = 0; u < kBuildU; u++) v[u] = d[u] >= 0 ? __ldg(rowof + d[u]) : 0u;
        bool dup = false;
#pragma unroll
        for (int u = 0; u < kBuildU; u++) {
            const int64_t r = b0 + (int64_t)u * blockDim.x + threadIdx.x;
            if (d[u] < 0) continue;
            if ((v[u] & kRowMask) != (uint32_t)r) {
                dup = true;
                continue;
            }
            const uint32_t meta = 1u | (((v[u] >> kRowBits) & 3u) << 1);
            vg_st256(P.pay + d[u], (uint64_t)jt.dmin + (uint64_t)d[u],
                     (unsigned long long)(uint32_t)r | ((unsigned long long)meta << 32), p0[u], p1[u]);
        }
        if (__any_sync(0xFFFFFFFFu, dup) && (threadIdx.x & 31) == 0) atomicOr(counters + 3, 1u);
    }
}

// The entries of keys no build row has (and the extra entry at cap): absent.
__global__ void jt_pay_absent_kernel(VgJoinTable jt, const uint32_t *rowof, PayArgs P) {
    const int64_t step = (int64_t)gridDim.x * blockDim.x * kBuildU;
    for (int64_t b0 = (int64_t)blockIdx.x * blockDim.x * kBuildU; b0 <= jt.cap; b0 += step) {
        uint32_t v[kBuildU];
#pragma unroll
        for (int u = 0; u < kBuildU; u++) {
            const int64_t d = b0 + (int64_t)u * blockDim.x + threadIdx.x;
            v[u] = d < jt.cap ? __ldg(rowof + d) : 0xFFFFFFFFu;
        }
#pragma unroll
        for (int u = 0; u < kBuildU; u++) {
            const int64_t d = b0 + (int64_t)u * blockDim.x + threadIdx.x;
            if (d <= jt.cap && v[u] == 0xFFFFFFFFu) vg_st256(P.pay + d, 0ull, 0ull, 0ull, 0ull);
        }
    }
}

// Compact entries by slot (coalesced writes): slot d takes the row its key
// recorded in pass 1 and that row's would-be entry, with the narrowed
// column rebased on its minimum; slots no row has are cleared.
// Also counts the slots some row recorded (counters[6]); with a payload
// that does not fit compact entries (statistics of pass 1) it only counts.
__global__ void jt_pay16_gather_kernel(VgJoinTable jt, const uint32_t *rowof, const ulonglong2 *payrow, int n_cols,
                                       int narrow, int narrow_type, const long long *mm, VgJPay16 *pay,
                                       uint32_t *counters) {
    long long nmin = 0;
    const bool fits = payrow && pay16_fits(n_cols, narrow, narrow_type, mm, &nmin);
    unsigned long long present = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d <= jt.cap; d += stride) {
        const uint32_t v = d < jt.cap ? __ldg(rowof + d) : 0xFFFFFFFFu;
        present += v != 0xFFFFFFFFu;
        if (!fits) continue;
        ulonglong2 e = make_ulonglong2(0ull, 0ull);
        if (v != 0xFFFFFFFFu) {
            const ulonglong2 q = __ldg(payrow + (v & kRowMask));
            const uint32_t meta = 1u | (((v >> kRowBits) & 3u) << 1);
            const uint32_t b = n_cols == 1 ? 0u : (uint32_t)q.y - (uint32_t)(unsigned long long)nmin;
            e = make_ulonglong2(q.x, (unsigned long long)b | ((unsigned long long)meta << 32));
        }
        *((ulonglong2 *)pay + d) = e;
    }
    for (int o = 16; o > 0; o >>= 1) present += __shfl_xor_sync(0xFFFFFFFFu, present, o);
    if ((threadIdx.x & 31) == 0 && present) atomicAdd((unsigned long long *)(counters + 6), present);
}

// The slot table of a unique-key direct table from its payload copy, for
// consumers that read slots (the general kernels, the join node's probe).
__global__ void jt_slots_from_pay_kernel(VgJoinTable jt, const VgJPay *pay) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= jt.cap; i += stride) {
        const ulonglong2 e = __ldg((const ulonglong2 *)(pay + i));
        const bool present = ((e.y >> 32) & 1u) != 0;
        *(ulonglong2 *)(jt.slots + i) =
            make_ulonglong2(present ? e.x : VG_JEMPTY, (e.y & 0xFFFFFFFFull) | ((present ? 1ull : 0ull) << 32));
    }
}

__global__ void jt_count_kernel(VgJoinTable jt, uint32_t *counters) {
    __shared__ unsigned s_nd, s_mx;
    if (threadIdx.x == 0) { s_nd = 0; s_mx = 0; }
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned nd = 0, mx = 0;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < jt.cap; s += stride) {
        const int32_t c = jt.slots[s].count;
        nd += c > 0;
        mx = (unsigned)c > mx ? (unsigned)c : mx;
    }
    nd = __reduce_add_sync(0xFFFFFFFFu, nd);
    mx = __reduce_max_sync(0xFFFFFFFFu, mx);
    if ((threadIdx.x & 31) == 0) {
        if (nd) atomicAdd(&s_nd, nd);
        if (mx) atomicMax(&s_mx, mx);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_nd) atomicAdd(counters + 0, s_nd);
        if (s_mx > 1) atomicMax(counters + 1, s_mx);
    }
}

// Payload copy of a direct table in build-row order: column reads are
// coalesced, each row writes its key's whole 32-byte entry (the entries
// start zeroed: absent keys read as not present).
__global__ void jt_pay_direct_kernel(VgJoinTable jt, VgCol key, VgCol c0, VgCol c1, int n_cols, VgJPay *pay) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= jt.n_build) return;
    if (!vg_valid(key, r)) return;
    const uint64_t k = vg_load_bits(key, r);
    const int64_t d = jt_direct_slot(jt, k);
    if (d < 0) return;
    uint64_t p0 = 0, p1 = 0;
    uint32_t meta = 1u;
    if (n_cols > 0) {
        p0 = vg_load_bits(c0, r);
        if (vg_valid(c0, r)) meta |= 2u;
    }
    if (n_cols > 1) {
        p1 = vg_load_bits(c1, r);
        if (vg_valid(c1, r)) meta |= 4u;
    }
    ulonglong2 *o = (ulonglong2 *)(pay + d);
    o[0] = make_ulonglong2(k, (unsigned long long)(uint32_t)r | ((unsigned long long)meta << 32));
    o[1] = make_ulonglong2(p0, p1);
}

__global__ void pair_keys_kernel(const int32_t *rslot, int64_t n, int64_t cap, uint64_t *keys,
                                 int32_t *vals) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        int32_t s = rslot[r];
        keys[r] = s < 0 ? (uint64_t)cap + 1 : (uint64_t)s;   // NA rows sort last
        vals[r] = (int32_t)r;
    }
}

__global__ void seg_start_kernel(VgJoinTable jt, const uint64_t *keys, int64_t n, int64_t nslots) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t k = keys[i];
        if (k >= (uint64_t)nslots) continue;
        if (i == 0 || keys[i - 1] != k) *jt_start_ptr(jt, (int64_t)k) = (int32_t)i;
    }
}

// ---------------------------------------------------------------------
// probe
// ---------------------------------------------------------------------
__global__ void probe_count_kernel(VgJoinTable jt, KeyArgs K, int64_t n_logical, const int32_t *sel,
                                   int kind, int32_t *cnt, int32_t *start, int32_t *flag) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t li = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; li < n_logical; li += stride) {
        int64_t p = sel ? (int64_t)sel[li] : li;
        uint64_t k[VG_MAX_KEYS];
        int32_t s0 = 0, c = 0;
        if (key_words(K, p, k) && jt_lookup(jt, k, s0, c)) {}
        else c = 0;
        start[li] = s0;
        switch (kind) {
        case JOIN_SEMI: cnt[li] = 0; flag[li] = c > 0; break;
        case JOIN_ANTI: cnt[li] = 0; flag[li] = c == 0; break;
        case JOIN_INNER: cnt[li] = c; flag[li] = 0; break;
        default: cnt[li] = c; flag[li] = c == 0; break;   // LEFT / FULL
        }
    }
}

__global__ void probe_emit_kernel(VgJoinTable jt, int64_t n_logical, const int32_t *sel, int kind,
                                  const int32_t *cnt, const int32_t *start, const int32_t *flag,
                                  const int64_t *off, const int64_t *off2, const int64_t *totals,
                                  int32_t *out_probe, int32_t *out_build, uint32_t *build_matched) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t matched_total = totals[0];
    for (int64_t li = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; li < n_logical; li += stride) {
        int32_t p = sel ? sel[li] : (int32_t)li;
        int32_t c = cnt[li];
        if (c > 0) {
            int64_t o = off[li];
            int32_t s0 = start[li];
            for (int32_t m = 0; m < c; m++) {
                // descending build row: the last of the ascending list first
                int64_t br = jt_row(jt, s0, c - 1 - m);
                out_probe[o + m] = p;
                out_build[o + m] = (int32_t)br;
                if (build_matched) atomicOr(build_matched + (br >> 5), 1u << (br & 31));
            }
        }
        if (flag[li]) {
            int64_t o = (kind == JOIN_SEMI || kind == JOIN_ANTI) ? off2[li] : matched_total + off2[li];
            out_probe[o] = p;
            if (out_build) out_build[o] = -1;
        }
    }
}

__global__ void unmatched_flags_kernel(const uint32_t *matched, int64_t n, int32_t *flag) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        flag[i] = !((matched[i >> 5] >> (i & 31)) & 1u);
}

__global__ void scatter_flags_kernel(const int32_t *flag, const int64_t *off, int64_t n, int32_t *out) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        if (flag[i]) out[off[i]] = (int32_t)i;
}

struct ProbeScratch {
    int32_t *cnt, *start, *flag;
    int64_t *off, *off2, *totals;
    void *scan;
    size_t scan_bytes;
};

bool carve_probe(void *base, size_t bytes, int64_t n, ProbeScratch &ps) {
    char *p = (char *)base;
    size_t o = 0;
    ps.cnt = (int32_t *)(p + o); o += a256((size_t)n * 4);
    ps.start = (int32_t *)(p + o); o += a256((size_t)n * 4);
    ps.flag = (int32_t *)(p + o); o += a256((size_t)n * 4);
    ps.off = (int64_t *)(p + o); o += a256((size_t)n * 8);
    ps.off2 = (int64_t *)(p + o); o += a256((size_t)n * 8);
    ps.totals = (int64_t *)(p + o); o += 256;
    ps.scan = p + o;
    ps.scan_bytes = vgk_scan_scratch(n);
    o += a256(ps.scan_bytes);
    return o <= bytes;
}

}  // namespace

extern "C" {

const char *vgk_join_last_error(void) { return g_err; }

int64_t vgk_join_cap(int64_t n_build) {
    int64_t cap = 64;
    while (cap * 3 < n_build * 4) cap <<= 1;   // load factor <= 3/4
    return cap;
}

size_t vgk_join_build_scratch_bytes(int64_t n_build) {
    int64_t n = n_build > 0 ? n_build : 1;
    // rows' slots, sort keys, sort scratch, counters, payload min / max
    // words, and the row of each key of a direct table (whose range is
    // below max(2 n, 65536), node_join.c)
    const size_t rowof = a256((size_t)((2 * n > 65536 ? 2 * n : 65536) + 64) * 4);
    return a256((size_t)n * 4) + a256((size_t)n * 8) + vgk_sort_pairs_scratch(n) + 256 + 256 + rowof +
           a256((size_t)n * 16);   // pass 1's row-order compact entries
}

// jt->cap, state, keys, start, count, rows (n_build entries) are allocated by
// the caller; on return jt->rows is NULL when every key is unique.
int vgk_join_build(VgJoinTable *jt, const VgCol *keys, int n_keys, const int32_t *key_conv,
                   int64_t n_build, void *d_scratch, size_t scratch_bytes, int64_t *h_distinct,
                   int64_t *h_maxdup, const VgCol *pay_cols, int n_pay, VgJPay *pay, int64_t *h_pay_mm,
                   int *h_pay_layout, int64_t *h_pay_min, int *slots_ready, vg_stream_t s) {
    if (h_pay_layout) *h_pay_layout = -2;
    if (h_pay_min) *h_pay_min = 0;
    cudaStream_t st = (cudaStream_t)s;
    if (scratch_bytes < vgk_join_build_scratch_bytes(n_build)) {
        snprintf(g_err, sizeof(g_err), "join build scratch too small");
        return -1;
    }
    int64_t n = n_build > 0 ? n_build : 1;
    char *p = (char *)d_scratch;
    int32_t *rslot = (int32_t *)p; p += a256((size_t)n * 4);
    uint64_t *pkeys = (uint64_t *)p; p += a256((size_t)n * 8);
    void *sort_scratch = p; p += vgk_sort_pairs_scratch(n);
    uint32_t *counters = (uint32_t *)p; p += 256;
    long long *mm = (long long *)p; p += 256;
    if (h_pay_mm)
        for (int i = 0; i < 6; i++) h_pay_mm[i] = 0;
    KeyArgs K;
    memset(&K, 0, sizeof(K));
    K.n_keys = n_keys;
    for (int i = 0; i < n_keys; i++) {
        K.cols[i] = keys[i];
        K.conv[i] = key_conv[i];
        K.types[i] = jt->key_types[i];
    }
    PayArgs P;
    memset(&P, 0, sizeof(P));
    if (pay && jt->direct && jt->slots && n_keys == 1 && n_pay >= 0 && n_pay <= 2) {
        P.pay = pay;
        P.n_cols = n_pay;
        if (n_pay > 0) P.c0 = pay_cols[0];
        if (n_pay > 1) P.c1 = pay_cols[1];
        // the column a compact entry would narrow: a bool or int64 one (the
        // second if both qualify)
        P.narrow = -1;
        if (n_pay == 2) {
            if (P.c1.type == VEC_INT64 || P.c1.type == VEC_BOOL) P.narrow = 1;
            else if (P.c0.type == VEC_INT64 || P.c0.type == VEC_BOOL) P.narrow = 0;
        }
    }
    if (slots_ready) *slots_ready = 1;
    if (P.pay && n_build >= ((int64_t)1 << kRowBits)) P.pay = nullptr;   // too many rows for rowof: no payload
    if (P.pay && ((uintptr_t)P.pay & 31u)) {
        snprintf(g_err, sizeof(g_err), "join build: payload copy not 32-byte aligned");
        return -1;
    }
    if (P.pay) {
        // direct table with a payload copy: rows record themselves per key,
        // then each recorded row writes its key's entry with its payload
        // values (a row whose key records another row reports a repeated
        // key) and the entries of absent keys are cleared; the slot table is
        // derived later, only if something reads it
        // (vgk_join_slots_from_payload)
        uint32_t *rowof = (uint32_t *)p;
        p += a256((size_t)((2 * n > 65536 ? 2 * n : 65536) + 64) * 4);
        // a payload that can take compact entries (one column, or a bool /
        // int64 one to narrow) also gets each row's would-be entry in row
        // order in pass 1, to be gathered by slot once the narrowed column's
        // range is known
        const bool cand16 = h_pay_layout && !getenv("VGPU_PAY32") && (n_pay == 1 || P.narrow >= 0);
        P.payrow = cand16 ? (ulonglong2 *)p : nullptr;
        jt_init_kernel<<<1, 32, 0, st>>>(*jt, counters, nullptr, 0, mm);
        vg_launch_counter++;
        if (check(cudaMemsetAsync(rowof, 0xFF, (size_t)jt->cap * 4, st), "join build")) return -1;
        vg_prof_begin(VG_PROF_JOIN_BUILD, st);
        const int ntype = P.narrow == 1 ? P.c1.type : P.c0.type;
        if (n_build > 0) {
            const int gb = grid_for((n_build + kBuildU - 1) / kBuildU, 256);
            jt_rows_direct_kernel<<<gb, 256, 0, st>>>(*jt, K, n_build, rslot, counters, P, rowof, mm);
            vg_launch_counter++;
        }
        // compact entries gathered by slot if the payload fits them (decided
        // on the device), and the slots present counted either way
        jt_pay16_gather_kernel<<<grid_for(jt->cap + 1, 256), 256, 0, st>>>(*jt, rowof, P.payrow, P.n_cols, P.narrow,
                                                                            ntype, mm, (VgJPay16 *)P.pay, counters);
        vg_launch_counter++;
        vg_prof_end(VG_PROF_JOIN_BUILD, st);
        // counters and the payload min / max words are adjacent (256 bytes
        // apart): one read-back
        long long hbuf[32 + 6];
        if (check(cudaMemcpyAsync(hbuf, counters, 256 + 48, cudaMemcpyDeviceToHost, st), "join build")) return -1;
        if (check(cudaStreamSynchronize(st), "join build")) return -1;
        uint32_t hc[8];
        memcpy(hc, hbuf, sizeof(hc));
        const long long *hm = hbuf + 32;
        if (hc[2]) {
            snprintf(g_err, sizeof(g_err), "join build: key outside the direct range (code %u)", hc[2]);
            return -1;
        }
        if (h_pay_mm)
            for (int i = 0; i < 6; i++) h_pay_mm[i] = hm[i];
        unsigned long long recorded = 0, present = 0;
        memcpy(&recorded, hc + 4, 8);
        memcpy(&present, hc + 6, 8);
        const bool repeated = present < recorded;
        long long nmin = 0;
        const bool fits16 = cand16 && pay16_fits(P.n_cols, P.narrow, ntype, hm, &nmin);
        if (!repeated) {
            if (fits16) {
                *h_pay_layout = P.n_cols == 1 ? -1 : P.narrow;
                if (h_pay_min) *h_pay_min = nmin;
            } else {
                // full entries: each recorded row writes its key's entry
                vg_prof_begin(VG_PROF_JOIN_BUILD, st);
                if (n_build > 0) {
                    const int gb = grid_for((n_build + kBuildU - 1) / kBuildU, 256);
                    jt_pay_scatter_kernel<<<gb, 256, 0, st>>>(*jt, rowof, rslot, n_build, P, counters);
                    vg_launch_counter++;
                }
                jt_pay_absent_kernel<<<grid_for((jt->cap + kBuildU) / kBuildU, 256), 256, 0, st>>>(*jt, rowof, P);
                vg_launch_counter++;
                vg_prof_end(VG_PROF_JOIN_BUILD, st);
            }
            if (check(cudaGetLastError(), "join build")) return -1;
            *h_distinct = -1;      // not counted on this path
            *h_maxdup = 1;
            jt->rows = nullptr;
            if (slots_ready) *slots_ready = 0;
            return 0;
        }
        P.pay = nullptr;   // a key repeats: the payload does not apply; build the slots by counting
    }
    { jt_init_kernel<<<grid_for(jt->cap + 1, 256), 256, 0, st>>>(*jt, counters, nullptr, 1, nullptr); vg_launch_counter++; }
    vg_prof_begin(VG_PROF_JOIN_BUILD, st);
    if (jt->direct) {
        if (n_build > 0) {
            jt_insert_direct_kernel<<<(unsigned)((n_build + 255) / 256), 256, 0, st>>>(*jt, K, n_build, rslot,
                                                                                  counters, P);
            vg_launch_counter++;
        }
        { jt_count_kernel<<<grid_for(jt->cap, 256), 256, 0, st>>>(*jt, counters); vg_launch_counter++; }
    } else {
        jt_insert_kernel<<<grid_for(n_build, 256), 256, 0, st>>>(*jt, K, n_build, rslot, counters);
        vg_launch_counter++;
    }
    vg_prof_end(VG_PROF_JOIN_BUILD, st);
    uint32_t hc[4] = {0, 0, 0, 0};
    cudaMemcpyAsync(hc, counters, 16, cudaMemcpyDeviceToHost, st);
    if (check(cudaStreamSynchronize(st), "join build")) return -1;
    if (hc[2]) {
        snprintf(g_err, sizeof(g_err), "join build: table overflow or wait expired (code %u)", hc[2]);
        return -1;
    }
    *h_distinct = hc[0];
    *h_maxdup = hc[1];
    if (hc[1] <= 1) {
        jt->rows = nullptr;    // start[slot] is the build row itself
        // hashed tables: the payload copy from the finished slots
        if (pay && !jt->direct && jt->slots) return vgk_join_payload(jt, nullptr, pay_cols, n_pay, pay, s);
        return 0;
    }
    // duplicates: stable sort of (slot, row) lays out each key's rows in
    // ascending row order
    int key_bits = 1;
    while (((int64_t)1 << key_bits) <= jt->cap + 1) key_bits++;
    { pair_keys_kernel<<<grid_for(n_build, 256), 256, 0, st>>>(rslot, n_build, jt->cap, pkeys, jt->rows); vg_launch_counter++; }
    if (vgk_sort_pairs(pkeys, jt->rows, n_build, key_bits, sort_scratch, vgk_sort_pairs_scratch(n), s)) {
        snprintf(g_err, sizeof(g_err), "%s", vgk_sort_last_error());
        return -1;
    }
    { seg_start_kernel<<<grid_for(n_build, 256), 256, 0, st>>>(*jt, pkeys, n_build, jt->slots ? jt->cap + 1 : jt->cap); vg_launch_counter++; }
    return check(cudaGetLastError(), "join build sort");
}

size_t vgk_join_probe_scratch_bytes(int64_t n_logical) {
    int64_t n = n_logical > 0 ? n_logical : 1;
    return a256((size_t)n * 4) * 3 + a256((size_t)n * 8) * 2 + 256 + a256(vgk_scan_scratch(n));
}

// Counts the output rows of one probe batch.  The per-row state stays in
// the scratch for vgk_join_probe_emit.
int vgk_join_probe_count(const VgJoinTable *jt, const VgCol *pkeys, int n_keys, const int32_t *key_conv,
                         int64_t n_rows, const int32_t *d_sel, int64_t sel_n, int kind,
                         void *d_scratch, size_t scratch_bytes, int64_t *h_total, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    int64_t n = d_sel ? sel_n : n_rows;
    ProbeScratch ps;
    if (!carve_probe(d_scratch, scratch_bytes, n > 0 ? n : 1, ps)) {
        snprintf(g_err, sizeof(g_err), "probe scratch too small");
        return -1;
    }
    if (n <= 0) { *h_total = 0; return 0; }
    KeyArgs K;
    memset(&K, 0, sizeof(K));
    K.n_keys = n_keys;
    for (int i = 0; i < n_keys; i++) {
        K.cols[i] = pkeys[i];
        K.conv[i] = key_conv[i];
        K.types[i] = jt->key_types[i];
    }
    vg_prof_begin(VG_PROF_JOIN_PROBE, st);
    { probe_count_kernel<<<grid_for(n, 256), 256, 0, st>>>(*jt, K, n, d_sel, kind, ps.cnt, ps.start, ps.flag); vg_launch_counter++; }
    vg_prof_end(VG_PROF_JOIN_PROBE, st);
    if (vgk_exclusive_scan(ps.cnt, n, ps.off, ps.totals + 0, ps.scan, ps.scan_bytes, s)) return -1;
    if (vgk_exclusive_scan(ps.flag, n, ps.off2, ps.totals + 1, ps.scan, ps.scan_bytes, s)) return -1;
    int64_t t[2] = {0, 0};
    cudaMemcpyAsync(t, ps.totals, 16, cudaMemcpyDeviceToHost, st);
    if (check(cudaStreamSynchronize(st), "probe count")) return -1;
    *h_total = t[0] + t[1];
    return 0;
}

int vgk_join_probe_emit(const VgJoinTable *jt, int64_t n_rows, const int32_t *d_sel, int64_t sel_n,
                        int kind, void *d_scratch, size_t scratch_bytes, int32_t *d_out_probe,
                        int32_t *d_out_build, uint32_t *d_build_matched, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    int64_t n = d_sel ? sel_n : n_rows;
    if (n <= 0) return 0;
    ProbeScratch ps;
    if (!carve_probe(d_scratch, scratch_bytes, n, ps)) {
        snprintf(g_err, sizeof(g_err), "probe scratch too small");
        return -1;
    }
    { probe_emit_kernel<<<grid_for(n, 256), 256, 0, st>>>(*jt, n, d_sel, kind, ps.cnt, ps.start, ps.flag,
                                                         ps.off, ps.off2, ps.totals, d_out_probe,
                                                         d_out_build, d_build_matched); vg_launch_counter++; }
    return check(cudaGetLastError(), "probe emit");
}

// FULL join: build rows never matched, in ascending order.
int vgk_join_unmatched_build(const uint32_t *d_matched, int64_t n_build, int32_t *d_out, int64_t *h_n,
                             void *d_scratch, size_t scratch_bytes, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    if (n_build <= 0) { *h_n = 0; return 0; }
    ProbeScratch ps;
    if (!carve_probe(d_scratch, scratch_bytes, n_build, ps)) {
        snprintf(g_err, sizeof(g_err), "unmatched scratch too small");
        return -1;
    }
    { unmatched_flags_kernel<<<grid_for(n_build, 256), 256, 0, st>>>(d_matched, n_build, ps.flag); vg_launch_counter++; }
    if (vgk_exclusive_scan(ps.flag, n_build, ps.off, ps.totals, ps.scan, ps.scan_bytes, s)) return -1;
    { scatter_flags_kernel<<<grid_for(n_build, 256), 256, 0, st>>>(ps.flag, ps.off, n_build, d_out); vg_launch_counter++; }
    int64_t t = 0;
    cudaMemcpyAsync(&t, ps.totals, 8, cudaMemcpyDeviceToHost, st);
    if (check(cudaStreamSynchronize(st), "unmatched build")) return -1;
    *h_n = t;
    return 0;
}

int vgk_join_payload(const VgJoinTable *jt, const VgCol *key, const VgCol *cols, int n_cols, VgJPay *pay,
                     vg_stream_t s) {
    if (!jt->slots || n_cols < 0 || n_cols > 2) {
        snprintf(g_err, sizeof(g_err), "join payload: unsupported table");
        return -1;
    }
    cudaStream_t st = (cudaStream_t)s;
    VgCol none;
    memset(&none, 0, sizeof(none));
    if (jt->direct && key) {
        if (check(cudaMemsetAsync(pay, 0, (size_t)(jt->cap + 1) * sizeof(VgJPay), st), "join payload")) return -1;
        if (jt->n_build > 0) {
            jt_pay_direct_kernel<<<(unsigned)((jt->n_build + 255) / 256), 256, 0, st>>>(
                *jt, *key, n_cols > 0 ? cols[0] : none, n_cols > 1 ? cols[1] : none, n_cols, pay);
            vg_launch_counter++;
        }
        return check(cudaGetLastError(), "join payload");
    }
    { jt_pay_kernel<<<grid_for(jt->cap + 1, 256), 256, 0, st>>>(*jt, n_cols > 0 ? cols[0] : none,
                                                             n_cols > 1 ? cols[1] : none, n_cols, pay);
      vg_launch_counter++; }
    return check(cudaGetLastError(), "join payload");
}

int vgk_join_slots_from_keys(const VgJoinTable *jt, const VgCol *key, int32_t key_conv, int64_t n_build,
                             void *d_scratch, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    KeyArgs K;
    memset(&K, 0, sizeof(K));
    K.n_keys = 1;
    K.cols[0] = *key;
    K.conv[0] = key_conv;
    K.types[0] = jt->key_types[0];
    PayArgs P;
    memset(&P, 0, sizeof(P));
    const int64_t n = n_build > 0 ? n_build : 1;
    int32_t *rslot = (int32_t *)d_scratch;
    uint32_t *counters = (uint32_t *)((char *)d_scratch + (((size_t)n * 4 + 127) & ~(size_t)127));
    jt_init_kernel<<<grid_for(jt->cap + 1, 256), 256, 0, st>>>(*jt, counters, nullptr, 1, nullptr);
    vg_launch_counter++;
    if (n_build > 0) {
        jt_insert_direct_kernel<<<(unsigned)((n_build + 255) / 256), 256, 0, st>>>(*jt, K, n_build, rslot, counters, P);
        vg_launch_counter++;
    }
    return check(cudaGetLastError(), "join slots");
}

int vgk_join_slots_from_payload(const VgJoinTable *jt, const VgJPay *pay, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    jt_slots_from_pay_kernel<<<grid_for(jt->cap + 1, 256), 256, 0, st>>>(*jt, pay);
    vg_launch_counter++;
    return check(cudaGetLastError(), "join slots");
}

}  // extern "C"
