// k_jit_pagg.cuh -- second step of the partitioned aggregation: the
// run-time specialised bucket reducer.
//
// The first step (vg_jit_agg in partition mode) has written every row with
// a valid int64 group key as a record (key, validity bits, the plan's
// distinct aggregate inputs) into the key-range bucket of its key; buckets
// are contiguous key ranges, ascending.  Here one CTA takes one bucket at a
// time, in bucket order from a ticket:
//   1. every record's key is looked up in a shared-memory hash table that
//      hands out dense group ids (all G groups' accumulators are
//      initialised when the bucket starts), and the record's values update
//      that group's accumulators with shared-memory atomics, in the same
//      representation as the fused kernel's cache (exact double sums as
//      32-bit digits in a window; a value outside the window goes to a
//      compensated pair in global memory);
//   2. the group ids are sorted by key (counting sort on the top bits of
//      the key's offset in the bucket's range, in shared memory);
//   3. each group's outputs are finished (the arithmetic of finish_kernel)
//      and written, in key order, to the staging area at stage_off[b].
// A bucket with more groups than one CTA holds is abandoned (ovf[b] = 1)
// and split further by the host.  Semantics: src/group_agg.c:155-281 and
// src/agg_ops.c:93-158, as for the other aggregation kernels.
//
// Included by the NVRTC source that jit_agg.cu generates, which defines
// before inclusion VGP_G (groups per CTA), VGP_S (hash slots), VGP_RW (record words),
// VGP_THREADS, VGP_MINB (CTAs per SM) and the layout offsets VGP_OFF_HID /
// VGP_OFF_GKEY, and after
// it the hooks vgp_init, vgp_acc and vgp_finish.

#pragma once
#include "k_groupby_dev.cuh"

namespace vgp {

constexpr uint32_t kEmptyId = 0xFFFFFFFFu;
constexpr uint32_t kBusyId = 0xFFFFFFFEu;
constexpr int G = VGP_G;
constexpr int S = VGP_S;          // hash slots: a power of two >= 2 G (load <= 1/2)
constexpr int RW = VGP_RW;
// key-order bins of the reducer's sort: the hash area (S >= 2 G words)
// holds the G ordered ids and then the bin counters
constexpr int kBins = (S - G) >= 2048 ? 2048 : (S - G) >= 1024 ? 1024 : (S - G) >= 512 ? 512 : 256;
constexpr int kBinBits = kBins == 2048 ? 11 : kBins == 1024 ? 10 : kBins == 512 ? 9 : 8;

// In-place exclusive scan of v[0..n) by the whole CTA (n a multiple of
// blockDim.x or smaller); wsum: 32 words of shared scratch.
VG_DEV void block_exclusive_scan(uint32_t *v, int n, uint32_t *wsum) {
    const int per = (n + (int)blockDim.x - 1) / (int)blockDim.x;
    const int lo = threadIdx.x * per;
    uint32_t t = 0;
    for (int i = 0; i < per; i++)
        if (lo + i < n) t += v[lo + i];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = t;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int nw = (int)(blockDim.x >> 5);
        uint32_t w = lane < nw ? wsum[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) wsum[lane] = w;
    }
    __syncthreads();
    uint32_t run = (warp ? wsum[warp - 1] : 0u) + x - t;
    for (int i = 0; i < per; i++) {
        if (lo + i < n) {
            const uint32_t c = v[lo + i];
            v[lo + i] = run;
            run += c;
        }
    }
    __syncthreads();
}

// flags bits beyond those of the accumulators (bit0..4): the group's
// compensated pair in global memory is being / has been initialised
constexpr uint32_t kFbInit = 32u, kFbReady = 64u;

// A double outside the group's digit window: compensated sum in global
// memory at fpos (the group's staging position).  The first such value
// of a group zeroes the pair; the others wait (bounded) until it has.
VG_DEV void sum_fallback(double *fs, double *fc, uint32_t *flags, double x, uint32_t *err) {
    const uint32_t old = atomicOr(flags, kFbInit);
    if (!(old & kFbInit)) {
        *fs = 0.0;
        *fc = 0.0;
        __threadfence();
        atomicOr(flags, kFbReady);
    } else {
        int spins = 0;
        while (!(*(volatile uint32_t *)flags & kFbReady)) {
            if (++spins > VG_SPIN_LIMIT) { atomicOr(err, VG_ERR_WAIT); return; }
        }
        __threadfence();
    }
    fallback_add(fs, fc, x);
}

// Correctly rounded double sum of a group: window digits (lo, hi pairs,
// stride G) plus, when the group used it, the compensated pair, all added
// exactly and rounded once.
__device__ __noinline__ double sum_wide(const int64_t (&win)[kWin], int b, uint32_t special, const double *fs,
                                        const double *fc) {
    int64_t w[VG_LACC_WORDS];
    for (int i = 0; i < VG_LACC_WORDS; i++) w[i] = 0;
    if (b != kBaseUnset)
        for (int i = 0; i < kWin; i++) w[b + i] += win[i];
    const double fb[2] = {*fs, *fc};
    for (int j = 0; j < 2; j++) {
        const VgDigits d = vg_split_double(vg_f64_to_bits(fb[j]));
        special |= d.special;
        if (d.lo >= 0) {
            w[d.lo] += d.d0;
            w[d.lo + 1] += d.d1;
            if (d.lo + 2 < VG_LACC_WORDS) w[d.lo + 2] += d.d2;
        }
    }
    return vg_digits_to_double(w, VG_LACC_WORDS, special);
}

VG_DEV double sum_result(const char *sm, uint32_t OBASE, uint32_t OWIN, int g, uint32_t flags, const double *fs,
                         const double *fc) {
    const int b = ((const int32_t *)(sm + OBASE))[g];
    int64_t win[kWin];
    const uint32_t *wl = (const uint32_t *)(sm + OWIN);
    const int32_t *wh = (const int32_t *)(sm + OWIN + 4 * G * kWin);
#pragma unroll
    for (int i = 0; i < kWin; i++) win[i] = b != kBaseUnset ? pair_get(wl + i * G + g, wh + i * G + g) : 0;
    const uint32_t special = flags & (4u | 8u | 16u);
    if (flags & kFbReady) return sum_wide(win, b, special, fs, fc);
    if ((special & 4u) || (special & 24u) == 24u) return __longlong_as_double(0x7FF8000000000000ll);
    if (special & 8u) return __longlong_as_double(0x7FF0000000000000ll);
    if (special & 16u) return __longlong_as_double((long long)0xFFF0000000000000ull);
    if (b == kBaseUnset) return 0.0;
    return vg_window6_to_double(win, b);
}

// One output of group g (finish_kernel's arithmetic on the shared state).
template <int FIN, int CLS, int IN_TYPE, uint32_t OCNT, uint32_t OVAL, uint32_t OFLAGS, uint32_t OBASE, uint32_t OWIN>
VG_DEV double finish(const char *sm, int g, const double *fs, const double *fc, bool &ok, uint32_t *warn) {
    ok = true;
    const uint32_t cnt = (CLS == VG_ACC_COUNT_ALL || CLS == VG_ACC_COUNT_VALID || FIN == AGG_MEAN ||
                          FIN == AGG_COUNT || FIN == AGG_COUNT_STAR)
                             ? ((const uint32_t *)(sm + OCNT))[g]
                             : 0u;
    if (FIN == AGG_COUNT || FIN == AGG_COUNT_STAR) return (double)cnt;
    const uint32_t fl = ((const uint32_t *)(sm + OFLAGS))[g];
    if (fl & 1u) { ok = false; return 0.0; }
    if (FIN == AGG_SUM || FIN == AGG_MEAN) {
        double s;
        if (IN_TYPE == VEC_DOUBLE) {
            s = sum_result(sm, OBASE, OWIN, g, fl, fs, fc);
        } else {
            s = vg_i2f(pair_get((const uint32_t *)(sm + OVAL) + g, (const int32_t *)(sm + OVAL + 4 * G) + g));
        }
        if (FIN == AGG_SUM) return s;
        if (cnt == 0) return __longlong_as_double(0x7FF8000000000000ll);
        return __ddiv_rn(s, (double)cnt);
    }
    // min / max
    if (!(fl & 2u)) {
        atomicAdd(warn, 1u);
        return FIN == AGG_MIN ? __longlong_as_double(0x7FF0000000000000ll)
                              : __longlong_as_double((long long)0xFFF0000000000000ull);
    }
    if (fl & 4u) return __longlong_as_double(0x7FF8000000000000ll);
    const int64_t v = ((const int64_t *)(sm + OVAL))[g];
    if (IN_TYPE == VEC_DOUBLE) return vg_bits_to_f64(vg_unord(v));
    return vg_i2f(v);
}

// Record p (RW words): 32-byte streaming loads when records are a
// multiple of 4 words (every record 32-byte aligned), else 16-byte ones.
VG_DEV void load_record(const ulonglong2 *rec, uint64_t p, uint64_t (&w)[RW]) {
    const uint64_t *q = (const uint64_t *)rec + p * RW;
    int i = 0;
    if (RW % 4 == 0) {
#pragma unroll
        for (; i + 4 <= RW; i += 4) vg_ld256_cs(q + i, w[i], w[i + 1], w[i + 2], w[i + 3]);
    }
#pragma unroll
    for (; i < RW; i += 2) {
        const ulonglong2 a = __ldcs((const ulonglong2 *)(q + i));
        w[i] = a.x;
        w[i + 1] = a.y;
    }
}

// Group id of key; -1 when the CTA holds G groups already (the bucket
// overflows).
VG_DEV int find(char *sm, uint64_t key, int *s_ng, int *s_ovf, uint32_t *dead);

}  // namespace vgp

// hooks written by the generator
VG_DEV void vgp_init(char *sm, int g);
VG_DEV void vgp_acc(char *sm, int g, const uint64_t (&w)[VGP_RW], const VgPaggReduce &B, uint64_t fpos);
VG_DEV uint32_t vgp_finish(const char *sm, int g, const VgPaggReduce &B, uint64_t fpos, uint64_t opos);

namespace vgp {

// Nobody waits: a thread that finds no entry for its key takes a private
// group id first (with the other lanes of its warp that reach that point,
// one counter update; every id's accumulators were initialised when the
// bucket started), writes the group's key, and only then publishes the id
// into an empty slot with one CAS.  A thread
// that loses the CAS to the same key marks its private id dead (skipped
// when the groups are ordered) and uses the winner's; one that loses it to
// another key keeps its initialised id for the next empty slot.
VG_DEV int find(char *sm, uint64_t key, int *s_ng, int *s_ovf, uint32_t *dead) {
    uint32_t *hid = (uint32_t *)(sm + VGP_OFF_HID);
    uint64_t *gk = (uint64_t *)(sm + VGP_OFF_GKEY);
    uint32_t s = (uint32_t)vg_mix64(key) & (uint32_t)(S - 1);
    int mine = -1;
    for (int probe = 0; probe < S; probe++) {
        uint32_t v = *(volatile uint32_t *)(hid + s);
        if (v == kEmptyId) {
            if (mine < 0) {
                const uint32_t m = __activemask();
                const int lane = threadIdx.x & 31;
                const int leader = __ffs(m) - 1;
                int base = 0;
                if (lane == leader) base = atomicAdd(s_ng, __popc(m));
                base = __shfl_sync(m, base, leader);
                mine = base + __popc(m & ((1u << lane) - 1u));
                if (mine >= G) {
                    *(volatile int *)s_ovf = 1;
                    return -1;
                }
                gk[mine] = key;                           // (its accumulators start initialised)
                __threadfence_block();
            }
            const uint32_t prev = atomicCAS(hid + s, kEmptyId, (uint32_t)mine);
            if (prev == kEmptyId) return mine;
            v = prev;
        }
        __threadfence_block();
        if (*(volatile uint64_t *)(gk + v) == key) {
            if (mine >= 0) atomicOr(dead + (mine >> 5), 1u << (mine & 31));
            return (int)v;
        }
        s = (s + 1) & (uint32_t)(S - 1);
    }
    *(volatile int *)s_ovf = 1;
    return -1;
}

}  // namespace vgp

extern "C" __global__ void __launch_bounds__(VGP_THREADS, VGP_MINB) vg_jit_pagg(const __grid_constant__ VgPaggReduce B) {
    using namespace vgp;
    extern __shared__ __align__(16) char sm[];
    __shared__ int s_bucket, s_ng, s_ovf, s_crowded, s_live;
    __shared__ uint32_t s_wsum[32];
    __shared__ uint32_t s_dead[(G + 31) / 32];        // group ids lost to a racing insert of the same key
    uint32_t *hid = (uint32_t *)(sm + VGP_OFF_HID);
    const uint64_t *gk = (const uint64_t *)(sm + VGP_OFF_GKEY);
    for (;;) {
        if (threadIdx.x == 0) {
            s_bucket = B.bucket_base + (int)atomicAdd(B.ticket, 1u);
            s_ng = 0;
            s_ovf = 0;
        }
        for (int i = threadIdx.x; i < S; i += blockDim.x) hid[i] = kEmptyId;
        for (int i = threadIdx.x; i < (G + 31) / 32; i += blockDim.x) s_dead[i] = 0;
        for (int g = threadIdx.x; g < G; g += blockDim.x) vgp_init(sm, g);   // every group's accumulators, coalesced
        __syncthreads();
        const int b = s_bucket;
        if (b >= B.bucket_base + B.n_buckets) break;
        const uint64_t sbase = B.stage_off[b];
        // 1. records -> groups (two records per thread in flight)
        for (int r = 0; r < B.n_regions; r++) {
            const uint64_t lo = B.roff[r][b];
            const uint64_t e = B.rend[r][b], e2 = B.roff[r][b + 1];
            const uint64_t hi = e < e2 ? e : e2;      // never past the bucket's range
            const ulonglong2 *rec = (const ulonglong2 *)B.rec[r];
            for (uint64_t p = lo + 2 * (uint64_t)threadIdx.x; p < hi; p += 2 * (uint64_t)blockDim.x) {
                if (*(volatile int *)&s_ovf) break;
                uint64_t w0[RW], w1[RW];
                const bool two = p + 1 < hi;
                load_record(rec, p, w0);
                if (two) load_record(rec, p + 1, w1);
                if (!(w0[1] & VG_PAGG_HOLE)) {                 // holes: positions no row took
                    const int g0 = find(sm, w0[0], &s_ng, &s_ovf, s_dead);
                    if (g0 < 0) break;
                    vgp_acc(sm, g0, w0, B, sbase + (uint64_t)g0);
                }
                if (two && !(w1[1] & VG_PAGG_HOLE)) {
                    const int g1 = find(sm, w1[0], &s_ng, &s_ovf, s_dead);
                    if (g1 < 0) break;
                    vgp_acc(sm, g1, w1, B, sbase + (uint64_t)g1);
                }
            }
        }
        __syncthreads();
        if (s_ovf) {
            if (threadIdx.x == 0) {
                B.gc[b] = 0;
                B.ovf[b] = 1;
            }
            __syncthreads();
            continue;
        }
        // 2. group ids in key order, in the hash area: a counting sort on
        //    the top bits of each key's offset in the bucket's key range,
        //    insertion sort within a bin; a bitonic sort if some bin is
        //    crowded (keys outside the range the buckets were cut for)
        const int n_ids = s_ng;                           // ids handed out (<= G: no overflow)
        uint32_t *ord = hid;
        uint32_t *cnt = hid + G;                          // kBins counters after the ids
        const uint64_t lo = B.omin + ((uint64_t)b << B.shift);
        const int sh = B.shift > kBinBits ? B.shift - kBinBits : 0;
        auto bin_of = [&](uint32_t g) -> int {
            const uint64_t ow = gk[g] ^ 0x8000000000000000ull;
            const uint64_t d = ow < lo ? 0ull : ((ow - lo) >> sh);
            return d >= (uint64_t)kBins ? kBins - 1 : (int)d;
        };
        auto live = [&](int g) { return !((s_dead[g >> 5] >> (g & 31)) & 1u); };
        for (int i = threadIdx.x; i < kBins; i += blockDim.x) cnt[i] = 0;
        if (threadIdx.x == 0) {
            s_crowded = 0;
            s_live = 0;
        }
        __syncthreads();
        {
            unsigned c = 0;
            for (int g = threadIdx.x; g < n_ids; g += blockDim.x)
                if (live(g)) {
                    atomicAdd(cnt + bin_of((uint32_t)g), 1u);
                    c++;
                }
            c = __reduce_add_sync(0xFFFFFFFFu, c);
            if ((threadIdx.x & 31) == 0 && c) atomicAdd(&s_live, (int)c);
        }
        __syncthreads();
        const int n = s_live;
        block_exclusive_scan(cnt, kBins, s_wsum);
        for (int g = threadIdx.x; g < n_ids; g += blockDim.x)
            if (live(g)) ord[atomicAdd(cnt + bin_of((uint32_t)g), 1u)] = (uint32_t)g;
        __syncthreads();
        for (int i = threadIdx.x; i < kBins; i += blockDim.x) {
            const int e = (int)cnt[i], st = i ? (int)cnt[i - 1] : 0;
            if (e - st <= 1) continue;
            if (e - st > 32) {
                s_crowded = 1;
                continue;
            }
            for (int x = st + 1; x < e; x++) {
                const uint32_t v = ord[x];
                const int64_t kv = (int64_t)gk[v];
                int y = x - 1;
                while (y >= st && (int64_t)gk[ord[y]] > kv) {
                    ord[y + 1] = ord[y];
                    y--;
                }
                ord[y + 1] = v;
            }
        }
        __syncthreads();
        if (s_crowded) {
            // the live ids are ord[0..n) already (bin order); sort them outright
            int P2 = 1;
            while (P2 < n) P2 <<= 1;
            for (int i = n + threadIdx.x; i < P2; i += blockDim.x) ord[i] = kEmptyId;
            __syncthreads();
            for (int size = 2; size <= P2; size <<= 1) {
                for (int stride = size >> 1; stride > 0; stride >>= 1) {
                    for (int i = threadIdx.x; i < P2; i += blockDim.x) {
                        const int j = i ^ stride;
                        if (j <= i) continue;
                        const uint32_t x = ord[i], y = ord[j];
                        // padding sorts last; keys compare as signed int64
                        bool gt;
                        if (x == kEmptyId) gt = y != kEmptyId;
                        else if (y == kEmptyId) gt = false;
                        else gt = (int64_t)gk[x] > (int64_t)gk[y];
                        const bool up = (i & size) == 0;
                        if (gt == up) {
                            ord[i] = y;
                            ord[j] = x;
                        }
                    }
                    __syncthreads();
                }
            }
        }
        // 3. results in key order
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int g = (int)ord[i];
            const uint64_t opos = sbase + (uint64_t)i;
            B.st_key[opos] = gk[g];
            B.st_ok[opos] = vgp_finish(sm, g, B, sbase + (uint64_t)g, opos);
        }
        if (threadIdx.x == 0) {
            B.gc[b] = (uint32_t)n;
            B.ovf[b] = 0;
        }
        __syncthreads();
    }
}
