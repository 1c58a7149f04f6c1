// k_serve.cu -- a serving loop over device-resident tables (vgpu_server_*).
//
// Requests (filter -> count / exact sum, group_by(key) -> exact sum + n,
// semi / anti join of one table against another) arrive at any time.  The
// pump (vgpu_server_poll) runs the loop:
//   retire  waves whose completion event fired: their requests are done and
//           their memory returns to the budget;
//   admit   queued requests in arrival order while their estimated memory
//           (group table, outputs, selection vectors) fits the budget;
//   launch  the admitted requests not yet running as one wave on a free
//           stream: work items of at most kChunk rows from every request,
//           taken by persistent CTAs (one wave = three kernel launches).
// Waves on different streams overlap on the device, and requests that
// arrive while others run join the next wave: continuous batching.  The
// tables stay resident; the key set of a table used as a semi / anti join
// build side is built on first use and kept.
//
// NA semantics follow the reference (src/filter.c, src/group_agg.c,
// src/join.c): a filter keeps valid values above the threshold; the NA key
// is its own group, sums skip NA values (na.rm); NA keys never match, so
// anti joins keep them.

#include <cstdio>
#include <cstring>
#include <deque>
#include <unordered_map>
#include <vector>
#include "k_set_dev.cuh"

#include "vgpu.h"

extern "C" int vgk_col_minmax_i64(const VgCol *col, int64_t n, int64_t *d_out, int64_t *h_out, vg_stream_t s);

namespace {

constexpr int kSrvThreads = 512;
constexpr int64_t kChunk = 1 << 18;
constexpr int kMaxWave = 256;

struct Table {
    const long long *key;
    const uint32_t *key_valid;     // 4-byte aligned bitmaps (or NULL: all valid)
    const long long *val;
    const uint32_t *val_valid;
    int64_t n;
    JSlot *keyset;                 // distinct valid keys, built on first use as a build side ...
    int64_t keyset_cap;
    uint32_t *kbits;               // ... or, for keys within a range of at most 2^30, one bit per key
    int64_t kmin, krange;
    int64_t distinct;              // distinct valid keys (after the key set is built), else -1
};

// one request of a wave, as the kernels see it
struct Req {
    int32_t kind;
    int32_t pad;
    Table probe;                   // source / probe table
    Table build;                   // semi / anti build side
    double threshold;
    long long *facc;               // filter: the sum as VG_LACC_WORDS 32-bit digits in 64-bit words ...
    uint32_t *fflags;              // ... and its NaN / infinity bits
    GSlot *gt;                     // group: table (cap + 2 slots: marker key, NA key)
    int64_t cap;
    int32_t direct;                // group over a dense key range: slot = key - probe.kmin (cap = krange)
    int32_t pad_direct;
    int64_t max_groups;
    long long *out_key;
    uint8_t *out_key_valid;
    double *out_sum;
    long long *out_n;
    int32_t *out_sel;
    int64_t first_chunk;
    unsigned long long *rows;      // result row count (device)
    unsigned long long *kept;      // filter: rows kept (device)
};

struct WItem {
    int32_t req, chunk;
    int64_t lo, hi;
};

VG_DEV bool bit(const uint32_t *v, int64_t r) { return v == nullptr || ((__ldg(v + (r >> 5)) >> (r & 31)) & 1u); }

VG_DEV bool keyset_has(const Table &B, uint64_t k) {
    if (B.kbits) {
        const uint64_t d = k - (uint64_t)B.kmin;
        return d < (uint64_t)B.krange && ((__ldg(B.kbits + (d >> 5)) >> (d & 31)) & 1u);
    }
    return j_find(B.keyset, B.keyset_cap, k) >= 0;
}

// ---------------------------------------------------------------------
// wave kernels
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(kSrvThreads) srv_init_kernel(const Req *req, int n_req) {
    for (int i = blockIdx.x; i < n_req; i += gridDim.x) {
        const Req &R = req[i];
        if (R.gt) {
            for (int64_t s = threadIdx.x; s < R.cap + 2; s += blockDim.x) {
                GSlot &g = R.gt[s];
                g.key = kEmpty;
                g.cnt = 0;
                g.base = kBaseUnset;
                g.flags = 0;
                for (int w = 0; w < kWin; w++) g.win[w] = 0;
                g.fs = 0.0;
                g.fc = 0.0;
            }
        }
        if (R.facc)
            for (int w = threadIdx.x; w < VG_LACC_WORDS; w += blockDim.x) R.facc[w] = 0;
        if (threadIdx.x == 0) {
            if (R.fflags) *R.fflags = 0;
            *R.rows = 0;
            if (R.kept) *R.kept = 0;
        }
    }
}

// phase 1: filter sums, group aggregation, semi / anti match counts
__global__ void __launch_bounds__(kSrvThreads) srv_phase1_kernel(const Req *req, const WItem *items, int n_items,
                                                                 long long *chunk_cnt, uint32_t *ctr) {
    extern __shared__ __align__(16) char dsm[];
    __shared__ int item;
    __shared__ unsigned long long s_cnt;
    for (;;) {
        if (threadIdx.x == 0) { item = (int)atomicAdd(ctr + 0, 1u); s_cnt = 0; }
        __syncthreads();
        const int it = item;
        if (it >= n_items) return;
        const WItem W = items[it];
        const Req &R = req[W.req];
        const Table &T = R.probe;
        unsigned c = 0;
        if (R.kind == VGPU_SERVE_FILTER_SUM) {
            // One exact sum for the whole request: every thread adds its
            // values' 32-bit digits into a six-digit window of its own (in
            // registers, anchored at its first value); a value outside it,
            // and each window at the end of the item, go into the CTA's
            // full-range digit words in shared memory; the CTA's words are
            // added to the request's once per item.  No atomics on one
            // address from every row.
            long long *cw = (long long *)dsm;                // VG_LACC_WORDS words
            uint32_t *cfl = (uint32_t *)(cw + VG_LACC_WORDS);
            for (int w = threadIdx.x; w < VG_LACC_WORDS; w += blockDim.x) cw[w] = 0;
            if (threadIdx.x == 0) *cfl = 0;
            __syncthreads();
            int64_t win[kWin];
#pragma unroll
            for (int w = 0; w < kWin; w++) win[w] = 0;
            int base = -1;
            uint32_t special = 0;
            for (int64_t r = W.lo + threadIdx.x; r < W.hi; r += blockDim.x) {
                if (!bit(T.val_valid, r)) continue;
                const uint64_t b = (uint64_t)__ldg(T.val + r);
                const double x = vg_bits_to_f64(b);
                if (!(x > R.threshold)) continue;
                c++;
                const VgDigits d = vg_split_double(b);
                if (d.special) { special |= d.special; continue; }
                if (d.lo < 0) continue;
                if (base < 0) {
                    base = d.lo - 2;
                    if (base < 0) base = 0;
                    if (base > VG_LACC_WORDS - kWin) base = VG_LACC_WORDS - kWin;
                }
                const int rel = d.lo - base;
                if (rel >= 0 && rel + 3 <= kWin) {
#pragma unroll
                    for (int w = 0; w < kWin; w++)
                        win[w] += w == rel ? d.d0 : w == rel + 1 ? d.d1 : w == rel + 2 ? d.d2 : 0;
                } else {
                    atomicAdd((unsigned long long *)(cw + d.lo), (unsigned long long)d.d0);
                    atomicAdd((unsigned long long *)(cw + d.lo + 1), (unsigned long long)d.d1);
                    if (d.lo + 2 < VG_LACC_WORDS) atomicAdd((unsigned long long *)(cw + d.lo + 2), (unsigned long long)d.d2);
                }
            }
            if (base >= 0) {
#pragma unroll
                for (int w = 0; w < kWin; w++)
                    if (win[w]) atomicAdd((unsigned long long *)(cw + base + w), (unsigned long long)win[w]);
            }
            if (special) atomicOr(cfl, special);
            __syncthreads();
            for (int w = threadIdx.x; w < VG_LACC_WORDS; w += blockDim.x)
                if (cw[w]) atomicAdd((unsigned long long *)(R.facc + w), (unsigned long long)cw[w]);
            if (threadIdx.x == 0 && *cfl) atomicOr(R.fflags, *cfl);
        } else if (R.kind == VGPU_SERVE_GROUP_SUM) {
            // hot keys aggregate in the CTA's cache, the rest go straight to
            // the request's table; the cache is merged at the end of the item
            GCache &gc = *(GCache *)dsm;
            gc_reset(gc);
            __syncthreads();
            for (int64_t r = W.lo + threadIdx.x; r < W.hi; r += blockDim.x) {
                const bool kv = bit(T.key_valid, r);
                const uint64_t k = kv ? (uint64_t)__ldg(T.key + r) : 0;
                const bool vv = bit(T.val_valid, r);
                const uint64_t v = vv ? (uint64_t)__ldg(T.val + r) : 0;
                const int cs = kv ? gc_find(gc, k) : -1;
                if (cs >= 0) {
                    atomicAdd(&gc.cnt[cs], 1u);
                    if (!vv || gc_sum(gc, cs, v)) continue;
                }
                const int64_t s = !kv ? R.cap + 1 : R.direct ? (int64_t)(k - (uint64_t)T.kmin) : g_slot(R.gt, R.cap, k);
                if (s < 0) { atomicOr(ctr + 4, VG_ERR_FULL); continue; }
                if (cs < 0) atomicAdd(&R.gt[s].cnt, 1ull);
                if (vv) g_add(R.gt[s], v);
            }
            __syncthreads();
            for (int i = threadIdx.x; i < kGC; i += blockDim.x) {
                if (gc.state[i] != 2u) continue;
                const int64_t s = R.direct ? (int64_t)(gc.key[i] - (uint64_t)T.kmin) : g_slot(R.gt, R.cap, gc.key[i]);
                if (s < 0) { atomicOr(ctr + 4, VG_ERR_FULL); continue; }
                gc_merge(gc, i, R.gt[s]);
            }
        } else {
            const bool semi = R.kind == VGPU_SERVE_SEMI;
            for (int64_t r = W.lo + threadIdx.x; r < W.hi; r += blockDim.x) {
                const bool m = bit(T.key_valid, r) &&
                               keyset_has(R.build, (uint64_t)__ldg(T.key + r));
                if (m == semi) c++;
            }
        }
        c = __reduce_add_sync(0xFFFFFFFFu, c);
        if ((threadIdx.x & 31) == 0 && c) atomicAdd(&s_cnt, (unsigned long long)c);
        __syncthreads();
        if (threadIdx.x == 0 && s_cnt) {
            if (R.kind == VGPU_SERVE_FILTER_SUM) atomicAdd(R.kept, s_cnt);
            else atomicAdd(R.rows, s_cnt);
        }
        if (threadIdx.x == 0 && (R.kind == VGPU_SERVE_SEMI || R.kind == VGPU_SERVE_ANTI))
            chunk_cnt[R.first_chunk + W.chunk] = (long long)s_cnt;
        __syncthreads();
    }
}

// phase 2: group outputs, semi / anti selection vectors in row order,
// filter sums rounded
__global__ void __launch_bounds__(kSrvThreads) srv_phase2_kernel(const Req *req, const WItem *items, int n_items,
                                                                 const long long *chunk_cnt, uint32_t *ctr) {
    __shared__ int item;
    __shared__ long long s_base;
    __shared__ int warp_tot[kSrvThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (;;) {
        if (threadIdx.x == 0) item = (int)atomicAdd(ctr + 1, 1u);
        __syncthreads();
        const int it = item;
        if (it >= n_items) return;
        const WItem W = items[it];
        const Req &R = req[W.req];
        if (R.kind == VGPU_SERVE_FILTER_SUM) {
            if (threadIdx.x == 0) R.out_sum[0] = vg_digits_to_double((const int64_t *)R.facc, VG_LACC_WORDS, *R.fflags);
        } else if (R.kind == VGPU_SERVE_GROUP_SUM) {
            // output rows taken per warp (one counter update per 32 slots,
            // not one per group)
            for (int64_t s0 = W.lo; s0 < W.hi; s0 += blockDim.x) {
                const int64_t s = s0 + threadIdx.x;
                const bool has = s < W.hi && R.gt[s].cnt != 0;
                const unsigned m = __ballot_sync(0xFFFFFFFFu, has);
                unsigned long long ob = 0;
                if (lane == 0 && m) ob = atomicAdd(R.rows, (unsigned long long)__popc(m));
                ob = __shfl_sync(0xFFFFFFFFu, ob, 0);
                if (!has) continue;
                const GSlot &g = R.gt[s];
                const unsigned long long o = ob + (unsigned long long)__popc(m & ((1u << lane) - 1u));
                if ((int64_t)o >= R.max_groups) { atomicOr(ctr + 4, VG_ERR_FULL); continue; }
                const bool na = s == R.cap + 1;
                R.out_key[o] = na ? 0 : R.direct ? (long long)(R.probe.kmin + s) : (long long)g.key;
                R.out_key_valid[o] = na ? 0 : 1;
                R.out_sum[o] = g_sum(g);
                R.out_n[o] = (long long)g.cnt;
            }
        } else {
            const bool semi = R.kind == VGPU_SERVE_SEMI;
            const Table &T = R.probe;
            if (threadIdx.x == 0) {
                long long b = 0;
                for (int c = 0; c < W.chunk; c++) b += chunk_cnt[R.first_chunk + c];
                s_base = b;
            }
            __syncthreads();
            for (int64_t r0 = W.lo; r0 < W.hi; r0 += blockDim.x) {
                const int64_t r = r0 + threadIdx.x;
                bool keep = false;
                if (r < W.hi) {
                    const bool m = bit(T.key_valid, r) &&
                                   keyset_has(R.build, (uint64_t)__ldg(T.key + r));
                    keep = m == semi;
                }
                const unsigned bm = __ballot_sync(0xFFFFFFFFu, keep);
                if (lane == 0) warp_tot[wid] = __popc(bm);
                __syncthreads();
                int before = 0, total = 0;
                for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
                    if (w < wid) before += warp_tot[w];
                    total += warp_tot[w];
                }
                if (keep) R.out_sel[s_base + before + __popc(bm & ((1u << lane) - 1u))] = (int32_t)r;
                __syncthreads();
                if (threadIdx.x == 0) s_base += total;
                __syncthreads();
            }
        }
        __syncthreads();
    }
}

// the key set of a build table: its distinct valid keys
__global__ void srv_keyset_kernel(Table T, uint32_t *err) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < T.n; r += stride) {
        if (!bit(T.key_valid, r)) continue;
        const int64_t s = j_insert(T.keyset, T.keyset_cap, (uint64_t)__ldg(T.key + r));
        if (s < 0) { atomicOr(err, VG_ERR_FULL); continue; }
        T.keyset[s].row = 1;                       // present (the marker key's slot included)
    }
}

__global__ void srv_keybits_kernel(Table T) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < T.n; r += stride) {
        if (!bit(T.key_valid, r)) continue;
        const uint64_t d = (uint64_t)__ldg(T.key + r) - (uint64_t)T.kmin;
        if (d < (uint64_t)T.krange) atomicOr(T.kbits + (d >> 5), 1u << (d & 31));
    }
}

__global__ void srv_keybits_count_kernel(const uint32_t *w, int64_t n_words, unsigned long long *n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned long long c = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_words; i += stride) c += __popc(w[i]);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(n, c);
}

__global__ void srv_keyset_count_kernel(const JSlot *t, int64_t cap, unsigned long long *n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned c = 0;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s <= cap; s += stride) c += t[s].row >= 0;
    c = __reduce_add_sync(0xFFFFFFFFu, c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(n, (unsigned long long)c);
}

__global__ void srv_keyset_init_kernel(JSlot *t, int64_t cap) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s <= cap; s += stride) {
        t[s].key = kEmpty;
        t[s].row = -1;
    }
}

// ---------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------
struct Request {
    VgpuServeQuery q;
    int64_t id;
    int64_t bytes;                 // admission estimate (scratch + outputs)
    int64_t scratch_bytes;         // the part returned when the request finishes
    void *scratch;                 // group table (freed when the request finishes)
    int state;                     // 0 queued, 1 admitted, 2 running, 3 done
    void *mem;                     // outputs + scratch (device)
    Req dev;                       // kernel view (pointers into mem)
    unsigned long long h_rows = 0, h_kept = 0;
    double h_sum = 0.0;
};

struct Wave {
    cudaStream_t stream;
    cudaEvent_t done;
    std::vector<int64_t> ids;
    void *meta = nullptr;          // Req[] + items + chunk counts + counters (device)
    void *host = nullptr;          // pinned copy-back of the small results
    bool busy = false;
};

struct Server {
    std::vector<Table> tables;
    std::unordered_map<int64_t, Request> reqs;
    std::deque<int64_t> queue;     // queued, in arrival order
    std::vector<int64_t> ready;    // admitted, not yet launched
    std::vector<Wave> waves;
    int64_t budget = 0, used = 0, next_id = 0;
    int grid = 0;
    cudaStream_t build_stream = nullptr;
    uint32_t *d_err = nullptr;
    char err[256];
};

int srv_fail(Server *S, const char *fmt, const char *what) {
    snprintf(S->err, sizeof(S->err), fmt, what);
    return -1;
}

int64_t pow2_ge(int64_t x) {
    int64_t c = 64;
    while (c < x) c <<= 1;
    return c;
}

int ensure_keyset(Server *S, Table &T) {
    if (T.keyset || T.kbits) return 0;
    cudaStream_t bst = S->build_stream;
    // dense key ranges: a bitmap (fits L2 for ranges up to ~10^9 bits)
    if (T.n > 0) {
        VgCol kc;
        memset(&kc, 0, sizeof(kc));
        kc.type = VEC_INT64;
        kc.data = T.key;
        kc.valid = T.key_valid;
        int64_t mm[3];
        if (vgk_col_minmax_i64(&kc, T.n, (int64_t *)(S->d_err + 8), mm, (vg_stream_t)bst) != 0)
            return srv_fail(S, "server: %s", "key range failed");
        const uint64_t span = (uint64_t)mm[1] - (uint64_t)mm[0];
        if (mm[2] > 0 && span < ((uint64_t)1 << 30)) {
            T.kmin = mm[0];
            T.krange = (int64_t)span + 1;
            const int64_t words = (T.krange + 31) / 32;
            if (cudaMalloc(&T.kbits, (size_t)words * 4) != cudaSuccess)
                return srv_fail(S, "server: %s", "no device memory for a key bitmap");
            S->used += words * 4;
            cudaMemsetAsync(T.kbits, 0, (size_t)words * 4, bst);
            cudaMemsetAsync(S->d_err, 0, 16, bst);
            srv_keybits_kernel<<<S->grid, 256, 0, bst>>>(T);
            srv_keybits_count_kernel<<<S->grid, 256, 0, bst>>>(T.kbits, words, (unsigned long long *)(S->d_err + 2));
            vg_launch_counter += 2;
            uint32_t e[4] = {0, 0, 0, 0};
            cudaMemcpyAsync(e, S->d_err, 16, cudaMemcpyDeviceToHost, bst);
            if (cudaStreamSynchronize(bst) != cudaSuccess) return srv_fail(S, "server: %s", "key bitmap build failed");
            unsigned long long d = 0;
            memcpy(&d, e + 2, 8);
            T.distinct = (int64_t)d;
            return 0;
        }
    }
    T.keyset_cap = pow2_ge(2 * (T.n > 0 ? T.n : 1));
    if (cudaMalloc(&T.keyset, (size_t)(T.keyset_cap + 1) * sizeof(JSlot)) != cudaSuccess)
        return srv_fail(S, "server: %s", "no device memory for a join key set");
    S->used += (int64_t)(T.keyset_cap + 1) * (int64_t)sizeof(JSlot);
    cudaStream_t st = S->build_stream;
    srv_keyset_init_kernel<<<S->grid, 256, 0, st>>>(T.keyset, T.keyset_cap);
    cudaMemsetAsync(S->d_err, 0, 16, st);
    srv_keyset_kernel<<<S->grid, 256, 0, st>>>(T, S->d_err);
    srv_keyset_count_kernel<<<S->grid, 256, 0, st>>>(T.keyset, T.keyset_cap, (unsigned long long *)(S->d_err + 2));
    vg_launch_counter += 3;
    uint32_t e[4] = {0, 0, 0, 0};
    cudaMemcpyAsync(e, S->d_err, 16, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess || e[0]) return srv_fail(S, "server: %s", "key set build failed");
    unsigned long long d = 0;
    memcpy(&d, e + 2, 8);
    T.distinct = (int64_t)d;
    return 0;
}

// bytes a request holds while admitted (outputs and scratch)
// group table bytes of a request (scratch, released when it finishes)
// group table slots: the key range itself when the keys are dense (no
// hashing), else a power of two at least twice the distinct keys
int64_t group_cap(const Table &T) {
    if (T.kbits && T.krange <= 2 * (T.distinct + 1) + 1024) return T.krange;
    return pow2_ge(2 * (T.distinct + 1));
}

int64_t scratch_estimate(Server *S, const VgpuServeQuery &q) {
    if (q.kind != VGPU_SERVE_GROUP_SUM) return 0;
    const Table &T = S->tables[(size_t)q.table];
    return (group_cap(T) + 2) * (int64_t)sizeof(GSlot);
}

int64_t estimate(Server *S, const VgpuServeQuery &q) {
    const Table &T = S->tables[(size_t)q.table];
    switch (q.kind) {
    case VGPU_SERVE_FILTER_SUM: return 4096;
    case VGPU_SERVE_GROUP_SUM: {
        const int64_t g = T.distinct + 1;          // distinct keys + the NA group
        return (group_cap(T) + 2) * (int64_t)sizeof(GSlot) + g * (8 + 1 + 8 + 8) + 4096;
    }
    default:
        return T.n * 4 + ((T.n + kChunk - 1) / kChunk + 1) * 8 + 4096;
    }
}

int retire(Server *S) {
    for (auto &W : S->waves) {
        if (!W.busy || cudaEventQuery(W.done) != cudaSuccess) continue;
        const uint64_t *h = (const uint64_t *)W.host;
        if (h[3 * kMaxWave]) return srv_fail(S, "server: %s", "a group table was too small (wave error)");
        for (size_t i = 0; i < W.ids.size(); i++) {
            Request &R = S->reqs[W.ids[i]];
            R.h_rows = h[3 * i];
            R.h_kept = h[3 * i + 1];
            memcpy(&R.h_sum, &h[3 * i + 2], 8);
            R.state = 3;
            if (R.scratch) {                    // the group table is no longer needed
                cudaFreeAsync(R.scratch, W.stream);
                R.scratch = nullptr;
                S->used -= R.scratch_bytes;
                R.bytes -= R.scratch_bytes;
            }
        }
        cudaFreeAsync(W.meta, W.stream);
        W.meta = nullptr;
        W.busy = false;
        W.ids.clear();
    }
    return 0;
}

void admit(Server *S) {
    bool busy = !S->ready.empty();
    for (auto &W : S->waves) busy = busy || W.busy;
    while (!S->queue.empty()) {
        Request &R = S->reqs[S->queue.front()];
        // over the budget: wait for running work to return memory; with
        // nothing running, admit anyway (results the client still holds must
        // not stall the queue forever)
        if (S->used + R.bytes > S->budget && busy) break;
        busy = true;
        S->used += R.bytes;
        R.state = 1;
        S->ready.push_back(R.id);
        S->queue.pop_front();
    }
}

int launch(Server *S) {
    while (!S->ready.empty()) {
        Wave *W = nullptr;
        for (auto &w : S->waves)
            if (!w.busy) { W = &w; break; }
        if (!W) return 0;
        const size_t n = S->ready.size() < (size_t)kMaxWave ? S->ready.size() : (size_t)kMaxWave;
        std::vector<Req> reqs;
        std::vector<WItem> it1, it2;
        int64_t chunks = 0;
        for (size_t i = 0; i < n; i++) {
            Request &R = S->reqs[S->ready[i]];
            const Table &T = S->tables[(size_t)R.q.table];
            Req &D = R.dev;
            memset(&D, 0, sizeof(D));
            D.kind = R.q.kind;
            D.probe = T;
            D.threshold = R.q.threshold;
            // outputs and scratch of the request, one allocation on the wave's stream
            size_t bytes = 256 * 2;
            if (D.kind == VGPU_SERVE_GROUP_SUM) {
                D.cap = group_cap(T);
                D.direct = D.cap == T.krange && T.kbits ? 1 : 0;
                D.max_groups = T.distinct + 1;
                bytes += (size_t)D.max_groups * 25 + 1024;
                if (cudaMallocAsync(&R.scratch, (size_t)(D.cap + 2) * sizeof(GSlot), W->stream) != cudaSuccess)
                    return srv_fail(S, "server: %s", "device allocation failed");
                D.gt = (GSlot *)R.scratch;
            } else if (D.kind == VGPU_SERVE_FILTER_SUM) {
                bytes += VG_LACC_WORDS * 8 + 256;
            } else {
                D.build = S->tables[(size_t)R.q.build_table];
                bytes += (size_t)T.n * 4 + 256;
            }
            char *m = nullptr;
            if (cudaMallocAsync((void **)&m, bytes, W->stream) != cudaSuccess)
                return srv_fail(S, "server: %s", "device allocation failed");
            R.mem = m;
            D.rows = (unsigned long long *)m;
            D.kept = (unsigned long long *)(m + 8);
            D.out_sum = (double *)(m + 16);
            char *p = m + 512;
            if (D.kind == VGPU_SERVE_GROUP_SUM) {
                D.out_sum = (double *)p; p += D.max_groups * 8;
                D.out_key = (long long *)p; p += D.max_groups * 8;
                D.out_n = (long long *)p; p += D.max_groups * 8;
                D.out_key_valid = (uint8_t *)p;
                for (int64_t lo = 0; lo < T.n; lo += kChunk)
                    it1.push_back(WItem{(int32_t)i, 0, lo, lo + kChunk < T.n ? lo + kChunk : T.n});
                for (int64_t lo = 0; lo < D.cap + 2; lo += kChunk)
                    it2.push_back(WItem{(int32_t)i, 0, lo, lo + kChunk < D.cap + 2 ? lo + kChunk : D.cap + 2});
            } else if (D.kind == VGPU_SERVE_FILTER_SUM) {
                D.facc = (long long *)p;
                D.fflags = (uint32_t *)(p + VG_LACC_WORDS * 8);
                for (int64_t lo = 0; lo < T.n; lo += kChunk)
                    it1.push_back(WItem{(int32_t)i, 0, lo, lo + kChunk < T.n ? lo + kChunk : T.n});
                it2.push_back(WItem{(int32_t)i, 0, 0, 0});
            } else {
                D.out_sel = (int32_t *)p;
                D.first_chunk = chunks;
                int32_t c = 0;
                for (int64_t lo = 0; lo < T.n; lo += kChunk, c++) {
                    it1.push_back(WItem{(int32_t)i, c, lo, lo + kChunk < T.n ? lo + kChunk : T.n});
                    it2.push_back(WItem{(int32_t)i, c, lo, lo + kChunk < T.n ? lo + kChunk : T.n});
                    chunks++;
                }
            }
            R.state = 2;
            reqs.push_back(D);
        }
        // wave metadata: requests, work lists, chunk counts, counters
        const size_t a_req = ((sizeof(Req) * n) + 255) & ~(size_t)255;
        const size_t a_it1 = ((sizeof(WItem) * (it1.size() + 1)) + 255) & ~(size_t)255;
        const size_t a_it2 = ((sizeof(WItem) * (it2.size() + 1)) + 255) & ~(size_t)255;
        const size_t a_cc = ((size_t)8 * (chunks + 1) + 255) & ~(size_t)255;
        char *meta = nullptr;
        if (cudaMallocAsync((void **)&meta, a_req + a_it1 + a_it2 + a_cc + 256, W->stream) != cudaSuccess)
            return srv_fail(S, "server: %s", "device allocation failed");
        W->meta = meta;
        Req *d_req = (Req *)meta;
        WItem *d_it1 = (WItem *)(meta + a_req);
        WItem *d_it2 = (WItem *)(meta + a_req + a_it1);
        long long *d_cc = (long long *)(meta + a_req + a_it1 + a_it2);
        uint32_t *d_ctr = (uint32_t *)(meta + a_req + a_it1 + a_it2 + a_cc);
        cudaStream_t st = W->stream;
        cudaMemcpyAsync(d_req, reqs.data(), sizeof(Req) * n, cudaMemcpyHostToDevice, st);
        if (!it1.empty()) cudaMemcpyAsync(d_it1, it1.data(), sizeof(WItem) * it1.size(), cudaMemcpyHostToDevice, st);
        if (!it2.empty()) cudaMemcpyAsync(d_it2, it2.data(), sizeof(WItem) * it2.size(), cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(d_ctr, 0, 32, st);
        srv_init_kernel<<<S->grid, kSrvThreads, 0, st>>>(d_req, (int)n);
        srv_phase1_kernel<<<S->grid, kSrvThreads, sizeof(GCache), st>>>(d_req, d_it1, (int)it1.size(), d_cc, d_ctr);
        srv_phase2_kernel<<<S->grid, kSrvThreads, 0, st>>>(d_req, d_it2, (int)it2.size(), d_cc, d_ctr);
        vg_launch_counter += 3;
        // the small results (and the wave's error word) back to pinned host memory
        uint64_t *h = (uint64_t *)W->host;
        for (size_t i = 0; i < n; i++) {
            cudaMemcpyAsync(h + 3 * i, reqs[i].rows, 8, cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(h + 3 * i + 1, reqs[i].kept, 8, cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(h + 3 * i + 2, reqs[i].out_sum, 8, cudaMemcpyDeviceToHost, st);
        }
        h[3 * kMaxWave] = 0;
        cudaMemcpyAsync(h + 3 * kMaxWave, d_ctr + 4, 4, cudaMemcpyDeviceToHost, st);
        cudaEventRecord(W->done, st);
        if (cudaGetLastError() != cudaSuccess) return srv_fail(S, "server: %s", "wave launch failed");
        W->ids.assign(S->ready.begin(), S->ready.begin() + (long)n);
        W->busy = true;
        S->ready.erase(S->ready.begin(), S->ready.begin() + (long)n);
    }
    return 0;
}

}  // namespace

extern "C" {

void vg_set_error(const char *fmt, ...);

void *vgpu_server_create(int n_streams, int64_t budget_bytes) {
    if (n_streams < 1) n_streams = 1;
    Server *S = new Server();
    S->budget = budget_bytes > 0 ? budget_bytes : ((int64_t)120 << 30);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    S->grid = sms > 0 ? sms * 2 : 64;             // two CTAs per SM: two group caches fit
    cudaFuncSetAttribute(srv_phase1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GCache));
    S->waves.resize((size_t)n_streams);
    for (auto &W : S->waves) {
        if (cudaStreamCreateWithFlags(&W.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&W.done, cudaEventDisableTiming) != cudaSuccess ||
            cudaMallocHost(&W.host, (size_t)kMaxWave * 24 + 64) != cudaSuccess) {
            vg_set_error("vgpu_server_create: stream / event / pinned buffer creation failed");
            return nullptr;
        }
    }
    if (cudaStreamCreateWithFlags(&S->build_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&S->d_err, 256) != cudaSuccess) {
        vg_set_error("vgpu_server_create: setup failed");
        return nullptr;
    }
    return S;
}

int vgpu_server_add_table(void *srv, const int64_t *key, const uint8_t *key_valid, const double *val,
                          const uint8_t *val_valid, int64_t n) {
    Server *S = (Server *)srv;
    if (!S || n < 0 || (n > 0 && (!key || !val)) || ((uintptr_t)key_valid & 3) || ((uintptr_t)val_valid & 3)) {
        vg_set_error("vgpu_server_add_table: bad arguments");
        return -1;
    }
    Table T;
    memset(&T, 0, sizeof(T));
    T.key = (const long long *)key;
    T.key_valid = (const uint32_t *)key_valid;
    T.val = (const long long *)val;
    T.val_valid = (const uint32_t *)val_valid;
    T.n = n;
    T.distinct = -1;
    S->tables.push_back(T);
    return (int)S->tables.size() - 1;
}

int64_t vgpu_server_submit(void *srv, const VgpuServeQuery *q) {
    Server *S = (Server *)srv;
    if (!S || !q || q->table < 0 || q->table >= (int)S->tables.size() || q->kind < VGPU_SERVE_FILTER_SUM ||
        q->kind > VGPU_SERVE_ANTI ||
        ((q->kind == VGPU_SERVE_SEMI || q->kind == VGPU_SERVE_ANTI) &&
         (q->build_table < 0 || q->build_table >= (int)S->tables.size()))) {
        vg_set_error("vgpu_server_submit: bad query");
        return -1;
    }
    // the key set of the build side (joins) or of the table (group-by: its
    // distinct key count sizes the group table), built once and kept
    Table &KT = S->tables[(size_t)(q->kind == VGPU_SERVE_GROUP_SUM ? q->table : q->build_table)];
    if (q->kind != VGPU_SERVE_FILTER_SUM && ensure_keyset(S, KT) != 0) {
        vg_set_error("%s", S->err);
        return -1;
    }
    Request R;
    R.q = *q;
    R.bytes = estimate(S, *q);
    if (R.bytes > S->budget) {
        // admission is by estimated bytes: a request that alone exceeds the
        // budget could never be admitted without breaking it
        vg_set_error("vgpu_server_submit: the request needs an estimated %lld bytes, more than the server's "
                     "budget of %lld", (long long)R.bytes, (long long)S->budget);
        return -1;
    }
    R.id = S->next_id++;
    R.scratch_bytes = scratch_estimate(S, *q);
    R.scratch = nullptr;
    R.state = 0;
    R.mem = nullptr;
    S->reqs[R.id] = R;
    S->queue.push_back(R.id);
    return R.id;
}

int vgpu_server_poll(void *srv) {
    Server *S = (Server *)srv;
    if (retire(S) != 0) {
        vg_set_error("%s", S->err);
        return -1;
    }
    admit(S);
    if (launch(S) != 0) {
        vg_set_error("%s", S->err);
        return -1;
    }
    int pending = 0;
    for (auto &kv : S->reqs)
        if (kv.second.state != 3) pending++;
    return pending;
}

int vgpu_server_done(void *srv, int64_t id) {
    Server *S = (Server *)srv;
    auto it = S->reqs.find(id);
    return it != S->reqs.end() && it->second.state == 3;
}

int vgpu_server_result(void *srv, int64_t id, VgpuServeResult *out) {
    Server *S = (Server *)srv;
    auto it = S->reqs.find(id);
    if (it == S->reqs.end() || it->second.state != 3) {
        vg_set_error("vgpu_server_result: request %lld is not done", (long long)id);
        return -1;
    }
    const Request &R = it->second;
    memset(out, 0, sizeof(*out));
    if (R.q.kind == VGPU_SERVE_FILTER_SUM) {
        out->rows = (int64_t)R.h_kept;
        out->sum = R.h_sum;
    } else if (R.q.kind == VGPU_SERVE_GROUP_SUM) {
        out->rows = (int64_t)R.h_rows;
        out->key = (const int64_t *)R.dev.out_key;
        out->key_valid = R.dev.out_key_valid;
        out->group_sum = R.dev.out_sum;
        out->group_n = (const int64_t *)R.dev.out_n;
    } else {
        out->rows = (int64_t)R.h_rows;
        out->sel = R.dev.out_sel;
    }
    return 0;
}

int vgpu_server_cancel(void *srv, int64_t id) {
    Server *S = (Server *)srv;
    if (!S) {
        vg_set_error("vgpu_server_cancel: no server");
        return -1;
    }
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) {
        vg_set_error("vgpu_server_cancel: no request %lld", (long long)id);
        return -1;
    }
    if (it->second.state != 0) {
        vg_set_error("vgpu_server_cancel: request %lld is already admitted (release it once it is done)",
                     (long long)id);
        return -1;
    }
    for (auto q = S->queue.begin(); q != S->queue.end(); ++q)
        if (*q == id) {
            S->queue.erase(q);
            break;
        }
    S->reqs.erase(it);
    return 0;
}

void vgpu_server_release(void *srv, int64_t id) {
    Server *S = (Server *)srv;
    auto it = S->reqs.find(id);
    if (it == S->reqs.end() || it->second.state != 3) return;
    if (it->second.mem) cudaFreeAsync(it->second.mem, S->build_stream);   // its wave has completed
    S->used -= it->second.bytes;
    S->reqs.erase(it);
}

void vgpu_server_free(void *srv) {
    Server *S = (Server *)srv;
    if (!S) return;
    for (auto &W : S->waves) {
        if (W.stream) cudaStreamSynchronize(W.stream);
        if (W.meta) cudaFree(W.meta);
        if (W.host) cudaFreeHost(W.host);
        if (W.done) cudaEventDestroy(W.done);
        if (W.stream) cudaStreamDestroy(W.stream);
    }
    for (auto &kv : S->reqs)
        if (kv.second.mem) cudaFree(kv.second.mem);
    for (auto &kv : S->reqs)
        if (kv.second.scratch) cudaFree(kv.second.scratch);
    for (auto &T : S->tables) {
        if (T.keyset) cudaFree(T.keyset);
        if (T.kbits) cudaFree(T.kbits);
    }
    if (S->build_stream) cudaStreamDestroy(S->build_stream);
    if (S->d_err) cudaFree(S->d_err);
    delete S;
}

int vgpu_server_warm(void *srv, int table) {
    Server *S = (Server *)srv;
    if (!S || table < 0 || table >= (int)S->tables.size()) {
        vg_set_error("vgpu_server_warm: bad table");
        return -1;
    }
    if (ensure_keyset(S, S->tables[(size_t)table]) != 0) {
        vg_set_error("%s", S->err);
        return -1;
    }
    return 0;
}

int vgpu_copy_to_host(void *dst_host, const void *src_device, int64_t bytes) {
    if (bytes <= 0) return 0;
    const cudaError_t e = cudaMemcpy(dst_host, src_device, (size_t)bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        vg_set_error("vgpu_copy_to_host: %s", cudaGetErrorString(e));
        return -1;
    }
    return 0;
}

}  // extern "C"
