// k_groupby_dev.cuh -- device helpers of the grouped aggregation kernels
// (k_groupby.cu, k_groupby_fast.cu).  Hash grouped aggregation on sm_103a, fused with the filter
// and, for joins feeding an aggregate, with the hash-join probe.
//
// Replaces the reference's per-row loop hash -> find_or_insert ->
// agg_accum_feed (src/group_agg.c:195-233, src/hash.c:103-134,
// src/agg_ops.c:93-158) and its sort-then-scan variant
// (src/group_agg.c:466-585):
//  * each CTA keeps a small open-addressing table of the groups it sees in
//    shared memory and updates it with shared-memory atomics;
//  * groups that do not fit go straight to a global open-addressing table
//    in HBM, and every CTA merges its shared table into it at the end;
//  * double sums are accumulated EXACTLY as 32-bit fixed-point digits in
//    64-bit integer words (integer atomics only; GB300's FP64 rate is a
//    small fraction of its integer rate), and rounded once at the end, so
//    every double sum and mean is the correctly rounded result;
//  * counts, integer sums (two's complement wrap, like the reference's
//    int64 arithmetic), min and max are exact integer atomics.
//
// The launch description lives in the constant bank (__grid_constant__) and
// the shared-memory layout is computed once per CTA, so the per-row path
// keeps everything in registers.

#pragma once
#ifndef __CUDACC_RTC__
#include <cstdio>
#include <cstring>
#endif
#include "k_common.cuh"

namespace {

#ifndef __CUDACC_RTC__
char g_err[256];
int check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof(g_err), "%s: %s", what, cudaGetErrorString(e));
        return -1;
    }
    return 0;
}
#endif

constexpr int kWin = 6;               // window digits per double sum
constexpr int kBaseUnset = 0x7FFFFFFF;
constexpr int kThreads = 512;
constexpr int kCacheProbes = 16;
constexpr int kGlobalProbes = 512;    // a longer probe means the table is too full: spill

__host__ __device__ inline bool acc_is_min(int cls) { return cls == VG_ACC_MIN_I64 || cls == VG_ACC_MIN_F64; }
__host__ __device__ inline bool acc_is_max(int cls) { return cls == VG_ACC_MAX_I64 || cls == VG_ACC_MAX_F64; }
__host__ __device__ inline bool has_val(int cls) {
    return cls == VG_ACC_SUM_I64 || cls == VG_ACC_MIN_I64 || cls == VG_ACC_MAX_I64 ||
           cls == VG_ACC_MIN_F64 || cls == VG_ACC_MAX_F64;
}

// values flowing into accumulators
struct InVal { uint64_t bits; bool ok; };

// ---------------------------------------------------------------------
// accumulator state of one table (shared cache, spill area or global)
// ---------------------------------------------------------------------
struct AccPtrs {
    uint64_t *cnt;      // count
    int64_t *val;       // int sum / min / max / ordered double image
    uint32_t *flags;    // bit0 has_na, bit1 has_value, bit2 NaN, bit3 +inf, bit4 -inf
    int32_t *base;      // window base digit (double sums)
    int64_t *win;       // [kWin][stride] window digits
    double *fs, *fc;    // compensated fallback sum (global table only)
};

// Layout of a cache-format area with `slots` slots (struct of arrays).
struct Lay {
    uint64_t state, nm, keys, first, total;
    uint64_t cnt[VG_MAX_ACCS], val[VG_MAX_ACCS], flags[VG_MAX_ACCS], base[VG_MAX_ACCS], win[VG_MAX_ACCS];
};

__host__ __device__ inline uint64_t al8(uint64_t x) { return (x + 7) & ~(uint64_t)7; }

__host__ __device__ inline void make_lay(const VgAggLaunch &L, uint64_t S, Lay &c) {
    uint64_t off = 0;
    c.state = off; off = al8(off + 4 * S);
    c.nm = off; off = al8(off + 4 * S);
    c.keys = off; off = al8(off + 8 * S * (uint64_t)L.n_keys);
    c.first = off; off = al8(off + (L.track_first ? 8 * S : 0));
    for (int a = 0; a < L.n_accs; a++) {
        int cls = L.acc[a].cls;
        c.cnt[a] = off; off = al8(off + 4 * S);
        c.val[a] = off; off = al8(off + (has_val(cls) ? 8 * S : 0));
        c.flags[a] = off; off = al8(off + 4 * S);
        c.base[a] = off; off = al8(off + (cls == VG_ACC_SUM_F64 ? 4 * S : 0));
        c.win[a] = off; off = al8(off + (cls == VG_ACC_SUM_F64 ? 8 * S * kWin : 0));
    }
    c.total = off;
}

// Cache-format state (shared-memory cache and spill area).  Shared memory
// has fast native 32-bit atomics but emulates 64-bit adds, so 64-bit
// quantities are kept as (u32 lo, i32 hi) word pairs: value = hi * 2^32 + lo,
// with carries / borrows of lo applied to hi, which is exact.
struct CPtrs {
    uint32_t *cnt;      // count
    uint32_t *vlo;      // int sum, low words (val pair) ...
    int32_t *vhi;       // ... and high words; min/max use the pair as one int64
    int64_t *val64;
    uint32_t *flags;
    int32_t *base;
    uint32_t *wlo;      // [kWin][S] window digits, low words
    int32_t *whi;       // [kWin][S] window digits, high words
};

VG_DEV CPtrs cptrs(char *base, const Lay &c, int a, int64_t S) {
    CPtrs p;
    p.cnt = (uint32_t *)(base + c.cnt[a]);
    p.vlo = (uint32_t *)(base + c.val[a]);
    p.vhi = (int32_t *)(base + c.val[a] + 4 * S);
    p.val64 = (int64_t *)(base + c.val[a]);
    p.flags = (uint32_t *)(base + c.flags[a]);
    p.base = (int32_t *)(base + c.base[a]);
    p.wlo = (uint32_t *)(base + c.win[a]);
    p.whi = (int32_t *)(base + c.win[a] + 4 * S * kWin);
    return p;
}

// adds a signed 64-bit value to a (lo, hi) pair with 32-bit atomics
VG_DEV void pair_add(uint32_t *lo, int32_t *hi, int64_t v) {
    uint32_t vl = (uint32_t)(uint64_t)v;
    int32_t vh = (int32_t)(v >> 32);      // v = vh * 2^32 + vl
    if (vl) {
        uint32_t old = atomicAdd(lo, vl);
        if ((uint32_t)(old + vl) < old) vh += 1;   // carry out of the low word
    }
    if (vh) atomicAdd(hi, vh);
}

VG_DEV int64_t pair_get(const uint32_t *lo, const int32_t *hi) {
    return (int64_t)(((uint64_t)(int64_t)*hi << 32) + (uint64_t)*lo);
}

// Double-sum state of the global table lives in lacc[a]:
//   [0, cap) int32 bases (in the first cap int64 words), then the window
//   digits [kWin][cap], then fs[cap], fc[cap].
VG_DEV AccPtrs global_ptrs(const VgGroupTable &gt, int a) {
    AccPtrs p;
    p.cnt = gt.cnt[a];
    p.val = gt.val[a];
    p.flags = gt.flags[a];
    int64_t *l = gt.lacc[a];
    p.base = (int32_t *)l;
    p.win = l + gt.cap;
    p.fs = (double *)(l + gt.cap * (1 + kWin));
    p.fc = p.fs + gt.cap;
    return p;
}

// ---------------------------------------------------------------------
// exact window accumulation
// ---------------------------------------------------------------------
// Adds the digits of d into the window of a slot.  Returns false when the
// value falls outside the window (the caller then uses a wider store).
VG_DEV bool win_add(int32_t *base_p, int64_t *win, int64_t stride, const VgDigits &d) {
    int b = *(volatile int *)base_p;
    if (b == kBaseUnset) {
        int want = d.lo - 2;
        if (want < 0) want = 0;
        if (want > VG_LACC_WORDS - kWin) want = VG_LACC_WORDS - kWin;
        int prev = atomicCAS((int *)base_p, kBaseUnset, want);
        b = (prev == kBaseUnset) ? want : prev;
    }
    int rel = d.lo - b;
    int need = d.d2 ? 3 : 2;
    if (rel < 0 || rel + need > kWin) return false;
    unsigned long long *w = (unsigned long long *)win;
    if (d.d0) atomicAdd(w + (int64_t)rel * stride, (unsigned long long)d.d0);
    if (d.d1) atomicAdd(w + (int64_t)(rel + 1) * stride, (unsigned long long)d.d1);
    if (d.d2) atomicAdd(w + (int64_t)(rel + 2) * stride, (unsigned long long)d.d2);
    return true;
}

// Compensated fallback: the atomic returns the previous sum, so the
// rounding error of this addition is recovered exactly with TwoSum
// (Knuth) and accumulated in a second word.
VG_DEV void fallback_add(double *s, double *c, double x) {
    double old = atomicAdd(s, x);
    double sum = __dadd_rn(old, x);
    double bp = __dsub_rn(sum, old);
    double e = __dadd_rn(__dsub_rn(old, __dsub_rn(sum, bp)), __dsub_rn(x, bp));
    if (e != 0.0) atomicAdd(c, e);
}

VG_DEV void set_flags(uint32_t *f, uint32_t bits) {
    uint32_t cur = *(volatile uint32_t *)f;
    if ((cur & bits) != bits) atomicOr(f, bits);
}

// Window add for the cache: digits into (lo, hi) pairs.  False when the
// value falls outside the window.
VG_DEV bool cwin_add(int32_t *base_p, uint32_t *wlo, int32_t *whi, int64_t S, const VgDigits &d) {
    int b = *(volatile int *)base_p;
    if (b == kBaseUnset) {
        int want = d.lo - 2;
        if (want < 0) want = 0;
        if (want > VG_LACC_WORDS - kWin) want = VG_LACC_WORDS - kWin;
        int prev = atomicCAS((int *)base_p, kBaseUnset, want);
        b = (prev == kBaseUnset) ? want : prev;
    }
    int rel = d.lo - b;
    int need = d.d2 ? 3 : 2;
    if (rel < 0 || rel + need > kWin) return false;
    if (d.d0) pair_add(wlo + (int64_t)rel * S, whi + (int64_t)rel * S, d.d0);
    if (d.d1) pair_add(wlo + (int64_t)(rel + 1) * S, whi + (int64_t)(rel + 1) * S, d.d1);
    if (d.d2) pair_add(wlo + (int64_t)(rel + 2) * S, whi + (int64_t)(rel + 2) * S, d.d2);
    return true;
}

// One input value into accumulator A of cache slot `slot`; false if the
// value must go to the global table instead (outside the window).
VG_DEV bool cache_update(const VgAccSpec &A, const CPtrs &P, int64_t S, int64_t slot, InVal x) {
    const int cls = A.cls;
    if (cls == VG_ACC_COUNT_ALL) { atomicAdd(P.cnt + slot, 1u); return true; }
    if (cls == VG_ACC_COUNT_VALID) { if (x.ok) atomicAdd(P.cnt + slot, 1u); return true; }
    if (!x.ok) {
        if (!A.na_rm) set_flags(P.flags + slot, 1u);
        return true;
    }
    switch (cls) {
    case VG_ACC_SUM_I64:
        atomicAdd(P.cnt + slot, 1u);
        pair_add(P.vlo + slot, P.vhi + slot, (int64_t)x.bits);
        return true;
    case VG_ACC_SUM_F64: {
        VgDigits d = vg_split_double(x.bits);
        if (d.special) set_flags(P.flags + slot, d.special);
        else if (d.lo >= 0 && !cwin_add(P.base + slot, P.wlo + slot, P.whi + slot, S, d)) return false;
        atomicAdd(P.cnt + slot, 1u);
        return true;
    }
    case VG_ACC_MIN_I64:
        atomicMin((long long *)(P.val64 + slot), (long long)x.bits);
        set_flags(P.flags + slot, 2u);
        return true;
    case VG_ACC_MAX_I64:
        atomicMax((long long *)(P.val64 + slot), (long long)x.bits);
        set_flags(P.flags + slot, 2u);
        return true;
    case VG_ACC_MIN_F64:
    case VG_ACC_MAX_F64:
        if (vg_is_nan_bits(x.bits)) { set_flags(P.flags + slot, 2u | 4u); return true; }
        if (cls == VG_ACC_MIN_F64) atomicMin((long long *)(P.val64 + slot), (long long)vg_ord(x.bits));
        else atomicMax((long long *)(P.val64 + slot), (long long)vg_ord(x.bits));
        set_flags(P.flags + slot, 2u);
        return true;
    default:
        return true;
    }
}

// One input value into accumulator A of a slot.  kGlobal selects the
// global table's fallback for values outside the window; in a cache the
// update is refused instead (returns false) and retried globally.
template <bool kGlobal>
VG_DEV bool acc_update(const VgAccSpec &A, const AccPtrs &P, int64_t stride, int64_t slot, InVal x) {
    const int cls = A.cls;
    if (cls == VG_ACC_COUNT_ALL) {
        atomicAdd((unsigned long long *)(P.cnt + slot), 1ull);
        return true;
    }
    if (cls == VG_ACC_COUNT_VALID) {
        if (x.ok) atomicAdd((unsigned long long *)(P.cnt + slot), 1ull);
        return true;
    }
    if (!x.ok) {
        if (!A.na_rm) set_flags(P.flags + slot, 1u);
        return true;
    }
    switch (cls) {
    case VG_ACC_SUM_I64:
        atomicAdd((unsigned long long *)(P.cnt + slot), 1ull);
        atomicAdd((unsigned long long *)(P.val + slot), (unsigned long long)x.bits);
        return true;
    case VG_ACC_SUM_F64: {
        VgDigits d = vg_split_double(x.bits);
        if (d.special) set_flags(P.flags + slot, d.special);
        else if (d.lo >= 0 && !win_add(P.base + slot, P.win + slot, stride, d)) {
            if (!kGlobal) return false;
            fallback_add(P.fs + slot, P.fc + slot, vg_bits_to_f64(x.bits));
        }
        atomicAdd((unsigned long long *)(P.cnt + slot), 1ull);
        return true;
    }
    case VG_ACC_MIN_I64:
        atomicMin((long long *)(P.val + slot), (long long)x.bits);
        set_flags(P.flags + slot, 2u);
        return true;
    case VG_ACC_MAX_I64:
        atomicMax((long long *)(P.val + slot), (long long)x.bits);
        set_flags(P.flags + slot, 2u);
        return true;
    case VG_ACC_MIN_F64:
    case VG_ACC_MAX_F64:
        if (vg_is_nan_bits(x.bits)) { set_flags(P.flags + slot, 2u | 4u); return true; }
        if (cls == VG_ACC_MIN_F64) atomicMin((long long *)(P.val + slot), (long long)vg_ord(x.bits));
        else atomicMax((long long *)(P.val + slot), (long long)vg_ord(x.bits));
        set_flags(P.flags + slot, 2u);
        return true;
    default:   // VG_ACC_NA_ONLY: only NA poisoning (bool min / max)
        return true;
    }
}

// ---------------------------------------------------------------------
// keys
// ---------------------------------------------------------------------
struct Keys { uint64_t w[VG_MAX_KEYS]; };
struct KeyTypes { int32_t t[VG_MAX_KEYS]; };

VG_DEV uint64_t hash_k(const Keys &k, int nk, uint32_t nm) {
    uint64_t h = 0x9E3779B97F4A7C15ull ^ nm;
#pragma unroll
    for (int i = 0; i < VG_MAX_KEYS; i++)
        if (i < nk) h = vg_mix64(h ^ k.w[i]) + (uint64_t)i;
    return vg_mix64(h);
}

VG_DEV bool keys_eq(const uint64_t *tk, int64_t stride, int64_t slot, const Keys &k, int nk,
                    const KeyTypes &kt, uint32_t tnm, uint32_t nm) {
    if (tnm != nm) return false;
#pragma unroll
    for (int i = 0; i < VG_MAX_KEYS; i++) {
        if (i >= nk) break;
        if ((nm >> i) & 1u) continue;   // both NA in this component
        uint64_t a = *(volatile const uint64_t *)(tk + (int64_t)i * stride + slot);
        if (!vg_key_word_eq(a, k.w[i], kt.t[i])) return false;
    }
    return true;
}

// Global table: returns the slot, or -1 when the table is too full (the
// caller spills and the host grows the table) or a bounded wait expired
// (err set).
VG_DEV int64_t gt_find_insert(const VgGroupTable &gt, const Keys &k, int nk, const KeyTypes &kt,
                              uint32_t nm, uint64_t h) {
    const int64_t mask = gt.cap - 1;
    int64_t slot = (int64_t)(h & (uint64_t)mask);
    const int64_t max_probe = gt.cap < kGlobalProbes ? gt.cap : kGlobalProbes;
    for (int64_t probe = 0; probe < max_probe; probe++) {
        // state 2 is published after the key words (fence + exchange), so
        // an acquire load of it orders the key reads below: no fence on the
        // lookup path
        uint32_t st = vg_ld_acquire(gt.state + slot);
        if (st == 0) {
            uint32_t prev = atomicCAS(gt.state + slot, 0u, 1u);
            if (prev == 0u) {
#pragma unroll
                for (int i = 0; i < VG_MAX_KEYS; i++)
                    if (i < nk) gt.keys[(int64_t)i * gt.cap + slot] = k.w[i];
                gt.nullmask[slot] = nm;
                __threadfence();
                atomicExch(gt.state + slot, 2u);
                atomicAdd(gt.n_used, 1u);
                return slot;
            }
            st = vg_ld_acquire(gt.state + slot);
        }
        st = vg_wait_while(gt.state + slot, 1u, st, VG_SPIN_LIMIT);
        if (st == 1u) { atomicOr(gt.err, VG_ERR_WAIT); return -1; }
        uint32_t tnm = *(volatile uint32_t *)(gt.nullmask + slot);
        if (keys_eq(gt.keys, gt.cap, slot, k, nk, kt, tnm, nm)) return slot;
        slot = (slot + 1) & mask;
    }
    return -1;
}

// ---------------------------------------------------------------------
// operands, values, predicate terms, join probe
// ---------------------------------------------------------------------
VG_DEV InVal load_operand(const VgOperand &o, const VgCol *pc, const VgCol *bc, int64_t pr, int64_t br) {
    InVal v;
    switch (o.side) {
    case VG_SIDE_PROBE: {
        const VgCol &c = pc[o.col];
        v.ok = vg_valid(c, pr);
        v.bits = vg_load_bits(c, pr);
        return v;
    }
    case VG_SIDE_BUILD: {
        if (br < 0) { v.ok = false; v.bits = 0; return v; }
        const VgCol &c = bc[o.col];
        v.ok = vg_valid(c, br);
        v.bits = vg_load_bits(c, br);
        return v;
    }
    case VG_SIDE_LIT:
        v.ok = true; v.bits = (uint64_t)o.lit; return v;
    default:
        v.ok = false; v.bits = 0; return v;
    }
}

VG_DEV uint64_t as_f64_bits(uint64_t bits, int type) {
    if (type == VEC_DOUBLE) return bits;
    return vg_f64_to_bits(vg_i2f((int64_t)bits));   // int64 or bool (0/1)
}

VG_DEV InVal eval_value(const VgValue &V, const VgCol *pc, const VgCol *bc, int64_t pr, int64_t br) {
    InVal a = load_operand(V.a, pc, bc, pr, br);
    if (V.op == 0) return a;
    InVal b = load_operand(V.b, pc, bc, pr, br);
    InVal r;
    r.ok = a.ok && b.ok;
    r.bits = 0;
    if (!r.ok) return r;
    if (V.type == VEC_DOUBLE) {
        double x = vg_bits_to_f64(as_f64_bits(a.bits, V.a.type));
        double y = vg_bits_to_f64(as_f64_bits(b.bits, V.b.type));
        double z;
        switch (V.op) {
        case '+': z = __dadd_rn(x, y); break;
        case '-': z = __dsub_rn(x, y); break;
        case '*': z = __dmul_rn(x, y); break;   // one rounding, never fused
        case '/': z = __ddiv_rn(x, y); break;
        default: z = fmod(x, y); break;
        }
        r.bits = vg_f64_to_bits(z);
    } else {
        int64_t x = (int64_t)a.bits, y = (int64_t)b.bits;
        uint64_t ux = (uint64_t)x, uy = (uint64_t)y;
        switch (V.op) {
        case '+': r.bits = ux + uy; break;
        case '-': r.bits = ux - uy; break;
        case '*': r.bits = ux * uy; break;
        case '/':
            if (y == 0) { r.ok = false; break; }
            r.bits = (y == -1) ? (0 - ux) : (uint64_t)(x / y);
            break;
        default:
            if (y == 0) { r.ok = false; break; }
            r.bits = (y == -1) ? 0 : (uint64_t)(x % y);
            break;
        }
    }
    return r;
}

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

VG_DEV bool probe_key_words(const VgAggLaunch &L, int64_t pr, uint64_t *k) {
#pragma unroll
    for (int i = 0; i < VG_MAX_KEYS; i++) {
        if (i >= L.n_jkeys) break;
        const VgCol &c = L.pcols[L.jkey_col[i]];
        if (!vg_valid(c, pr)) return false;            // NA never matches
        uint64_t b = vg_load_bits(c, pr);
        if (L.jkey_conv[i]) b = vg_f64_to_bits(vg_i2f((int64_t)b));
        int t = L.jt.key_types[i];
        if (t == VEC_DOUBLE && vg_is_nan_bits(b)) return false;
        k[i] = vg_norm_key(b, t);
    }
    return true;
}

// ---------------------------------------------------------------------
// cache entry merge / spill (shared by the kernel tail and the replay)
// ---------------------------------------------------------------------

// Merges cache-layout entry i (area `base`, layout c, stride S) into the
// global table.  Returns false if the global table had no room.
VG_DEV KeyTypes key_types(const VgAggLaunch &L) {
    KeyTypes kt;
#pragma unroll
    for (int i = 0; i < VG_MAX_KEYS; i++) kt.t[i] = i < L.n_keys ? L.key[i].type : 0;
    return kt;
}

VG_DEV bool merge_entry(const VgAggLaunch &L, char *base, const Lay &c, int64_t S, int64_t i) {
    const KeyTypes kt = key_types(L);
    Keys k;
    const uint64_t *sk = (const uint64_t *)(base + c.keys);
#pragma unroll
    for (int j = 0; j < VG_MAX_KEYS; j++) k.w[j] = j < L.n_keys ? sk[(int64_t)j * S + i] : 0;
    uint32_t nm = ((const uint32_t *)(base + c.nm))[i];
    uint64_t h = hash_k(k, L.n_keys, nm);
    int64_t g = gt_find_insert(L.gt, k, L.n_keys, kt, nm, h);
    if (g < 0) return false;
    if (L.track_first)
        atomicMin((unsigned long long *)(L.gt.first_row + g), ((unsigned long long *)(base + c.first))[i]);
    for (int a = 0; a < L.n_accs; a++) {
        const int cls = L.acc[a].cls;
        CPtrs sp = cptrs(base, c, a, S);
        AccPtrs gp = global_ptrs(L.gt, a);
        if (sp.cnt[i]) atomicAdd((unsigned long long *)(gp.cnt + g), (unsigned long long)sp.cnt[i]);
        uint32_t f = sp.flags[i];
        if (f) atomicOr(gp.flags + g, f);
        if (cls == VG_ACC_SUM_I64) {
            int64_t v = pair_get(sp.vlo + i, sp.vhi + i);
            if (v) atomicAdd((unsigned long long *)(gp.val + g), (unsigned long long)v);
        } else if (acc_is_min(cls)) {
            if (f & 2u) atomicMin((long long *)(gp.val + g), (long long)sp.val64[i]);
        } else if (acc_is_max(cls)) {
            if (f & 2u) atomicMax((long long *)(gp.val + g), (long long)sp.val64[i]);
        } else if (cls == VG_ACC_SUM_F64) {
            int bs = sp.base[i];
            if (bs == kBaseUnset) continue;
            // each digit word goes into the global window; words that do not
            // fit go through the compensated fallback, split into two
            // exactly representable halves
            int bg = *(volatile int *)(gp.base + g);
            if (bg == kBaseUnset) {
                int prev = atomicCAS((int *)(gp.base + g), kBaseUnset, bs);
                bg = (prev == kBaseUnset) ? bs : prev;
            }
            for (int w = 0; w < kWin; w++) {
                int64_t v = pair_get(sp.wlo + (int64_t)w * S + i, sp.whi + (int64_t)w * S + i);
                if (!v) continue;
                int rel = bs + w - bg;
                if (rel >= 0 && rel < kWin) {
                    atomicAdd((unsigned long long *)(gp.win + (int64_t)rel * L.gt.cap + g), (unsigned long long)v);
                } else {
                    int e = 32 * (bs + w) - 1074;
                    double hi = ldexp((double)(v >> 32), e + 32);
                    double lo = ldexp((double)(v & 0xFFFFFFFFll), e);
                    if (hi != 0.0) fallback_add(gp.fs + g, gp.fc + g, hi);
                    if (lo != 0.0) fallback_add(gp.fs + g, gp.fc + g, lo);
                }
            }
        }
    }
    return true;
}

// Copies cache entry i into the spill area (same layout, stride spill cap).
VG_DEV void spill_entry(const VgAggLaunch &L, char *sm, const Lay &c, int64_t S, int64_t i, const Lay &sl) {
    uint32_t j = atomicAdd(L.spill_cache_n, 1u);
    if ((int64_t)j >= L.spill_cache_cap) { atomicOr(L.gt.err, VG_ERR_SPILL); return; }
    const int64_t T = L.spill_cache_cap;
    char *d = L.spill_cache;
    ((uint32_t *)(d + sl.state))[j] = 2u;
    ((uint32_t *)(d + sl.nm))[j] = ((const uint32_t *)(sm + c.nm))[i];
    for (int k = 0; k < L.n_keys; k++)
        ((uint64_t *)(d + sl.keys))[(int64_t)k * T + j] = ((const uint64_t *)(sm + c.keys))[(int64_t)k * S + i];
    if (L.track_first) ((uint64_t *)(d + sl.first))[j] = ((const uint64_t *)(sm + c.first))[i];
    for (int a = 0; a < L.n_accs; a++) {
        CPtrs sp = cptrs(sm, c, a, S);
        CPtrs dp = cptrs(d, sl, a, T);
        dp.cnt[j] = sp.cnt[i];
        dp.flags[j] = sp.flags[i];
        int cls = L.acc[a].cls;
        if (cls == VG_ACC_SUM_I64) { dp.vlo[j] = sp.vlo[i]; dp.vhi[j] = sp.vhi[i]; }
        else if (has_val(cls)) dp.val64[j] = sp.val64[i];
        if (cls == VG_ACC_SUM_F64) {
            dp.base[j] = sp.base[i];
            for (int w = 0; w < kWin; w++) {
                dp.wlo[(int64_t)w * T + j] = sp.wlo[(int64_t)w * S + i];
                dp.whi[(int64_t)w * T + j] = sp.whi[(int64_t)w * S + i];
            }
        }
    }
}

VG_DEV void init_slot(const VgAggLaunch &L, char *base, const Lay &c, int64_t S, int64_t i) {
    ((uint32_t *)(base + c.state))[i] = 0;
    if (L.track_first) ((uint64_t *)(base + c.first))[i] = ~0ull;
    for (int a = 0; a < L.n_accs; a++) {
        CPtrs p = cptrs(base, c, a, S);
        p.cnt[i] = 0;
        p.flags[i] = 0;
        int cls = L.acc[a].cls;
        if (cls == VG_ACC_SUM_I64) { p.vlo[i] = 0; p.vhi[i] = 0; }
        else if (acc_is_min(cls)) p.val64[i] = 0x7FFFFFFFFFFFFFFFll;
        else if (acc_is_max(cls)) p.val64[i] = (int64_t)0x8000000000000000ull;
        if (cls == VG_ACC_SUM_F64) {
            p.base[i] = kBaseUnset;
            for (int w = 0; w < kWin; w++) { p.wlo[(int64_t)w * S + i] = 0; p.whi[(int64_t)w * S + i] = 0; }
        }
    }
}

VG_DEV bool spill_row(const VgAggLaunch &L, int64_t li, int32_t m, int acc) {
    uint32_t i = atomicAdd(L.spill_rows_n, 1u);
    if ((int64_t)i >= L.spill_rows_cap) { atomicOr(L.gt.err, VG_ERR_SPILL); return false; }
    L.spill_rows[2 * (int64_t)i] = li;
    L.spill_rows[2 * (int64_t)i + 1] = ((int64_t)m << 8) | (int64_t)(acc + 1);
    return true;
}

}  // namespace
