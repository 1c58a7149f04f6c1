// k_set_dev.cuh -- device building blocks shared by the query-set and the
// serving kernels (k_batch.cu, k_serve.cu): per-query group tables with
// exact double sums and per-query join / key-set tables, in global memory
// (small ones stay in L2 while their query runs).  Each query keeps the
// node path's semantics: groups and accumulators as in hash_agg_next_batch
// (src/group_agg.c:155-281) and agg_accum_feed (src/agg_ops.c:93-158),
// inner-join matches as in join_probe_one (src/join.c:262-480).
#pragma once
#include "k_groupby_dev.cuh"

namespace {

constexpr uint64_t kEmpty = 0x8000000000000000ull;    // free slot marker; that key has its own slot

// group table slot (array of structures: one group's state in two lines)
struct GSlot {
    unsigned long long key;
    unsigned long long cnt;
    int32_t base;             // digit window base, kBaseUnset until the first summand
    uint32_t flags;           // bit2 NaN, bit3 +inf, bit4 -inf
    long long win[kWin];      // digits of the exact sum (units of 2^-1074)
    double fs, fc;            // compensated fallback for summands outside the window
};

struct JSlot {
    unsigned long long key;
    long long row;
};

VG_DEV uint64_t bhash(uint64_t k) { return vg_mix64(k ^ 0x9E3779B97F4A7C15ull); }

// claims or finds key k's slot: index, or -1 when the table is full
VG_DEV int64_t g_slot(GSlot *t, int64_t cap, uint64_t k) {
    if (k == kEmpty) return cap;
    const int64_t mask = cap - 1;
    int64_t s = (int64_t)(bhash(k) & (uint64_t)mask);
    for (int64_t p = 0; p < cap; p++) {
        unsigned long long cur = *(volatile unsigned long long *)&t[s].key;
        if (cur == k) return s;
        if (cur == kEmpty) {
            const unsigned long long prev = atomicCAS(&t[s].key, kEmpty, k);
            if (prev == kEmpty || prev == k) return s;
        }
        s = (s + 1) & mask;
    }
    return -1;
}

// one double into slot g's exact sum
VG_DEV void g_add(GSlot &g, uint64_t bits) {
    const VgDigits d = vg_split_double(bits);
    if (d.special) { atomicOr(&g.flags, d.special); return; }
    if (d.lo < 0) return;
    int b = *(volatile int *)&g.base;
    if (b == kBaseUnset) {
        int want = d.lo - 2;
        if (want < 0) want = 0;
        if (want > VG_LACC_WORDS - kWin) want = VG_LACC_WORDS - kWin;
        const int prev = atomicCAS(&g.base, kBaseUnset, want);
        b = (prev == kBaseUnset) ? want : prev;
    }
    const int rel = d.lo - b;
    if (rel >= 0 && rel + (d.d2 ? 3 : 2) <= kWin) {
        if (d.d0) atomicAdd((unsigned long long *)&g.win[rel], (unsigned long long)d.d0);
        if (d.d1) atomicAdd((unsigned long long *)&g.win[rel + 1], (unsigned long long)d.d1);
        if (d.d2) atomicAdd((unsigned long long *)&g.win[rel + 2], (unsigned long long)d.d2);
    } else {
        fallback_add(&g.fs, &g.fc, vg_bits_to_f64(bits));
    }
}

// join slot of build key k (claimed); -1 when full
VG_DEV int64_t j_insert(JSlot *t, int64_t cap, uint64_t k) {
    if (k == kEmpty) return cap;
    const int64_t mask = cap - 1;
    int64_t s = (int64_t)(bhash(k) & (uint64_t)mask);
    for (int64_t p = 0; p < cap; p++) {
        const unsigned long long prev = atomicCAS(&t[s].key, kEmpty, k);
        if (prev == kEmpty || prev == k) return s;
        s = (s + 1) & mask;
    }
    return -1;
}

VG_DEV long long j_find(const JSlot *t, int64_t cap, uint64_t k) {
    if (k == kEmpty) return __ldg(&t[cap].row);
    const int64_t mask = cap - 1;
    int64_t s = (int64_t)(bhash(k) & (uint64_t)mask);
    for (int64_t p = 0; p < cap; p++) {
        const unsigned long long cur = __ldg(&t[s].key);
        if (cur == k) return __ldg(&t[s].row);
        if (cur == kEmpty) return -1;
        s = (s + 1) & mask;
    }
    return -1;
}

// exact sum of a group slot, rounded once
__device__ __noinline__ double g_sum_wide(const GSlot &g) {
    int64_t w[VG_LACC_WORDS];
    for (int i = 0; i < VG_LACC_WORDS; i++) w[i] = 0;
    if (g.base != kBaseUnset)
        for (int i = 0; i < kWin; i++) w[g.base + i] += g.win[i];
    uint32_t special = g.flags & (4u | 8u | 16u);
    const double fb[2] = {g.fs, g.fc};
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

// The correctly rounded sum of a slot: its window alone is rounded on
// registers (vg_window6_to_double); a slot that used the compensated pair
// or saw a NaN / infinity takes the general digit rounding.
static_assert(kWin == 6, "the register rounding takes a six-digit window");
VG_DEV double g_sum(const GSlot &g) {
    if (g.fs != 0.0 || g.fc != 0.0 || (g.flags & (4u | 8u | 16u))) return g_sum_wide(g);
    if (g.base == kBaseUnset) return 0.0;
    int64_t w[6];
#pragma unroll
    for (int i = 0; i < 6; i++) w[i] = g.win[i];
    return vg_window6_to_double(w, g.base);
}

}  // namespace

// ---------------------------------------------------------------------
// per-CTA shared-memory group cache for one work item: hot keys aggregate
// here (32-bit shared atomics) and reach their instance's table once per
// item instead of once per row
// ---------------------------------------------------------------------
namespace {

constexpr int kGC = 1024;                       // cache slots (power of two)

struct GCache {
    unsigned long long key[kGC];
    uint32_t state[kGC];                         // 0 empty, 1 being claimed, 2 ready
    uint32_t cnt[kGC];
    int32_t base[kGC];
    uint32_t flags[kGC];
    uint32_t wlo[kWin][kGC];
    int32_t whi[kWin][kGC];
    int used;
};

VG_DEV void gc_reset(GCache &c) {
    for (int i = threadIdx.x; i < kGC; i += blockDim.x) {
        c.state[i] = 0;
        c.cnt[i] = 0;
        c.base[i] = kBaseUnset;
        c.flags[i] = 0;
#pragma unroll
        for (int w = 0; w < kWin; w++) { c.wlo[w][i] = 0; c.whi[w][i] = 0; }
    }
    if (threadIdx.x == 0) c.used = 0;
}

// cache slot of key k, claimed if new and the cache is under 3/4 full; -1
// when the key is not cached
VG_DEV int gc_find(GCache &c, uint64_t k) {
    int s = (int)(bhash(k) & (uint64_t)(kGC - 1));
    // keys are cached while the cache is at most half full, so that a key
    // that is not cached (most keys of a high-cardinality table) is known to
    // be absent after a few probes: a linear probe at load 1/2 ends at an
    // empty slot after 2.5 probes on average
    const bool may_insert = *(volatile int *)&c.used < kGC / 2;
    for (int p = 0; p < (may_insert ? 8 : 4); p++) {
        uint32_t st = *(volatile uint32_t *)&c.state[s];
        if (st == 0) {
            if (!may_insert) return -1;
            const uint32_t prev = atomicCAS(&c.state[s], 0u, 1u);
            if (prev == 0u) {
                c.key[s] = k;
                __threadfence_block();
                atomicExch(&c.state[s], 2u);
                atomicAdd(&c.used, 1);
                return s;
            }
            st = prev;
        }
        int spins = 0;
        while (st == 1u) {
            if (++spins > VG_SPIN_LIMIT) return -1;
            st = *(volatile uint32_t *)&c.state[s];
        }
        __threadfence_block();
        if (*(volatile unsigned long long *)&c.key[s] == k) return s;
        s = (s + 1) & (kGC - 1);
    }
    return -1;
}

// a double into cache slot s's digit window; false: outside the window
VG_DEV bool gc_sum(GCache &c, int s, uint64_t bits) {
    const VgDigits32 d = vg_split_double32(bits);
    if (d.special) { atomicOr(&c.flags[s], d.special); return true; }
    if (d.zero) return true;
    int b = *(volatile int *)&c.base[s];
    if (b == kBaseUnset) {
        int want = d.word - 2;
        if (want < 0) want = 0;
        if (want > VG_LACC_WORDS - kWin) want = VG_LACC_WORDS - kWin;
        const int prev = atomicCAS(&c.base[s], kBaseUnset, want);
        b = (prev == kBaseUnset) ? want : prev;
    }
    const int rel = d.word - b;
    if (rel < 0 || rel + (d.d2 ? 3 : 2) > kWin) return false;
    const uint32_t dd[3] = {d.d0, d.d1, d.d2};
#pragma unroll
    for (int i = 0; i < 3; i++) {
        if (!dd[i]) continue;
        const uint32_t a = d.neg ? 0u - dd[i] : dd[i];
        const uint32_t o = atomicAdd(&c.wlo[rel + i][s], a);
        const bool carry = d.neg ? (o < dd[i]) : (o + a < o);
        if (carry) atomicAdd(&c.whi[rel + i][s], d.neg ? -1 : 1);
    }
    return true;
}

// cache slot s into global slot g (count, flags, digits)
VG_DEV void gc_merge(const GCache &c, int s, GSlot &g) {
    if (c.cnt[s]) atomicAdd(&g.cnt, (unsigned long long)c.cnt[s]);
    if (c.flags[s]) atomicOr(&g.flags, c.flags[s]);
    const int bs = c.base[s];
    if (bs == kBaseUnset) return;
    int bg = *(volatile int *)&g.base;
    if (bg == kBaseUnset) {
        const int prev = atomicCAS(&g.base, kBaseUnset, bs);
        bg = (prev == kBaseUnset) ? bs : prev;
    }
    for (int w = 0; w < kWin; w++) {
        const int64_t v = (int64_t)(((uint64_t)(int64_t)c.whi[w][s] << 32) + (uint64_t)c.wlo[w][s]);
        if (!v) continue;
        const int rel = bs + w - bg;
        if (rel >= 0 && rel < kWin) {
            atomicAdd((unsigned long long *)&g.win[rel], (unsigned long long)v);
        } else {
            // outside the table's window: two exactly representable halves
            // through the compensated fallback
            const int e = 32 * (bs + w) - 1074;
            const double hi = ldexp((double)(v >> 32), e + 32);
            const double lo = ldexp((double)(v & 0xFFFFFFFFll), e);
            if (hi != 0.0) fallback_add(&g.fs, &g.fc, hi);
            if (lo != 0.0) fallback_add(&g.fs, &g.fc, lo);
        }
    }
}

}  // namespace
