// k_groupby.cu -- hash grouped aggregation on sm_103a, fused with the filter
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

#include <cstdio>
#include <cstring>
#include "k_common.cuh"

namespace {

char g_err[256];
int check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof(g_err), "%s: %s", what, cudaGetErrorString(e));
        return -1;
    }
    return 0;
}

constexpr int kWin = 6;               // window digits per double sum
constexpr int kBaseUnset = 0x7FFFFFFF;
constexpr int kThreads = 512;
constexpr int kCacheProbes = 16;
constexpr int kGlobalProbes = 512;    // a longer probe means the table is too full: spill

VG_DEV bool acc_is_min(int cls) { return cls == VG_ACC_MIN_I64 || cls == VG_ACC_MIN_F64; }
VG_DEV bool acc_is_max(int cls) { return cls == VG_ACC_MAX_I64 || cls == VG_ACC_MAX_F64; }
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
        uint32_t st = *(volatile uint32_t *)(gt.state + slot);
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
            st = prev;
        }
        int spins = 0;
        while (st == 1u) {
            if (++spins > VG_SPIN_LIMIT) { atomicOr(gt.err, VG_ERR_WAIT); return -1; }
            __nanosleep(32);
            st = *(volatile uint32_t *)(gt.state + slot);
        }
        __threadfence();
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

// ---------------------------------------------------------------------
// the fused aggregation kernel
// ---------------------------------------------------------------------
template <bool kPred, bool kJoin, bool kCache>
__global__ void __launch_bounds__(kThreads, 2)
agg_kernel(const __grid_constant__ VgAggLaunch L, int64_t n_logical) {
    extern __shared__ __align__(16) char sm[];
    __shared__ Lay cl;
    __shared__ int cache_used;   // occupied cache slots; a nearly full cache stops taking new keys
    const int S = L.cache_slots;
    const int nk = L.n_keys;
    if (kCache) {
        if (threadIdx.x == 0) { make_lay(L, S, cl); cache_used = 0; }
        __syncthreads();
        for (int i = threadIdx.x; i < S; i += blockDim.x) init_slot(L, sm, cl, S, i);
        __syncthreads();
    }
    const bool replay = L.replay != nullptr;
    const KeyTypes kt = key_types(L);

    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < n_logical; it += stride) {
        int64_t li = it;
        int32_t m_lo = 0, m_hi = 0x7FFFFFFF;
        int only_acc = -1;
        if (replay) {
            li = L.replay[2 * it];
            int64_t w = L.replay[2 * it + 1];
            m_lo = (int32_t)(w >> 8);
            m_hi = m_lo + 1;
            only_acc = (int)(w & 0xFF) - 1;
        }
        const int64_t pr = L.sel ? (int64_t)L.sel[li] : li;
        if (kPred) {
            bool keep = true;
            for (int t = 0; t < L.pred.n_terms && keep; t++) keep = term_keep(L.pred.term[t], L.pcols, pr);
            if (!keep) continue;
        }
        int32_t mstart = 0, mcount = 1;
        bool matched = true;
        if (kJoin) {
            uint64_t jk[VG_MAX_KEYS];
            matched = probe_key_words(L, pr, jk) && jt_lookup(L.jt, jk, mstart, mcount);
            if (!matched) {
                if (L.join_kind != JOIN_LEFT) continue;
                mcount = 1;     // one output row with NA build columns
            }
        }
        if (m_hi > mcount) m_hi = mcount;
        for (int32_t m = m_lo; m < m_hi; m++) {
            int64_t br = -1;
            if (kJoin && matched) br = jt_row(L.jt, mstart, m);
            Keys k;
            uint32_t nm = 0;
#pragma unroll
            for (int i = 0; i < VG_MAX_KEYS; i++) {
                k.w[i] = 0;
                if (i < nk) {
                    InVal v = eval_value(L.key[i], L.pcols, L.bcols, pr, br);
                    if (!v.ok) nm |= 1u << i;
                    else k.w[i] = vg_norm_key(v.bits, L.key[i].type);
                }
            }
            uint64_t order = 0;
            if (L.track_first) {
                if (kJoin) {
                    // position in the join's output stream: batch, matched
                    // rows before unmatched, probe row, descending build row
                    uint64_t rank = matched ? (uint64_t)(mcount - 1 - m) : 0;
                    if (rank > 0x7FF) rank = 0x7FF;
                    order = ((uint64_t)L.batch_idx << 44) | ((uint64_t)(matched ? 0 : 1) << 43) |
                            ((uint64_t)(li & 0xFFFFFFFF) << 11) | rank;
                } else {
                    order = (uint64_t)(L.row_base + li);   // logical position in the stream
                }
            }
            const uint64_t h = hash_k(k, nk, nm);
            int found = -1;
            if (kCache) {
                uint32_t *st = (uint32_t *)(sm + cl.state);
                uint32_t *snm = (uint32_t *)(sm + cl.nm);
                uint64_t *sk = (uint64_t *)(sm + cl.keys);
                int slot = (int)(h & (uint64_t)(S - 1));
                const bool may_insert = *(volatile int *)&cache_used < (S * 3) / 4;
                for (int probe = 0; probe < (may_insert ? kCacheProbes : 4); probe++) {
                    uint32_t s0 = *(volatile uint32_t *)(st + slot);
                    if (s0 == 0) {
                        if (!may_insert) break;
                        uint32_t prev = atomicCAS(st + slot, 0u, 1u);
                        if (prev == 0u) {
#pragma unroll
                            for (int i = 0; i < VG_MAX_KEYS; i++)
                                if (i < nk) sk[(int64_t)i * S + slot] = k.w[i];
                            snm[slot] = nm;
                            __threadfence_block();
                            atomicExch(st + slot, 2u);
                            atomicAdd(&cache_used, 1);
                            found = slot;
                            break;
                        }
                        s0 = prev;
                    }
                    int spins = 0;
                    while (s0 == 1u) {
                        if (++spins > VG_SPIN_LIMIT) { atomicOr(L.gt.err, VG_ERR_WAIT); break; }
                        s0 = *(volatile uint32_t *)(st + slot);
                    }
                    if (s0 != 2u) break;
                    __threadfence_block();
                    if (keys_eq(sk, S, slot, k, nk, kt, *(volatile uint32_t *)(snm + slot), nm)) {
                        found = slot;
                        break;
                    }
                    slot = (slot + 1) & (S - 1);
                }
            }
            if (found >= 0) {
                if (L.track_first)
                    atomicMin((unsigned long long *)(sm + cl.first) + found, (unsigned long long)order);
                for (int a = 0; a < L.n_accs; a++) {
                    const VgAccSpec &A = L.acc[a];
                    InVal v = (A.cls == VG_ACC_COUNT_ALL) ? InVal{0, true}
                                                          : eval_value(A.in, L.pcols, L.bcols, pr, br);
                    if (cache_update(A, cptrs(sm, cl, a, S), S, found, v)) continue;
                    // value outside the shared window: this update goes to
                    // the global table
                    int64_t g = gt_find_insert(L.gt, k, nk, kt, nm, h);
                    if (g >= 0) acc_update<true>(A, global_ptrs(L.gt, a), L.gt.cap, g, v);
                    else spill_row(L, li, m, a);
                }
            } else {
                int64_t g = gt_find_insert(L.gt, k, nk, kt, nm, h);
                if (g < 0) { spill_row(L, li, m, only_acc); continue; }
                if (L.track_first && only_acc < 0)
                    atomicMin((unsigned long long *)(L.gt.first_row + g), (unsigned long long)order);
                for (int a = 0; a < L.n_accs; a++) {
                    if (only_acc >= 0 && only_acc != a) continue;
                    const VgAccSpec &A = L.acc[a];
                    InVal v = (A.cls == VG_ACC_COUNT_ALL) ? InVal{0, true}
                                                          : eval_value(A.in, L.pcols, L.bcols, pr, br);
                    acc_update<true>(A, global_ptrs(L.gt, a), L.gt.cap, g, v);
                }
            }
        }
    }

    if (!kCache) return;
    __syncthreads();
    __shared__ Lay sl;
    if (threadIdx.x == 0) make_lay(L, (uint64_t)L.spill_cache_cap, sl);
    __syncthreads();
    const uint32_t *st = (const uint32_t *)(sm + cl.state);
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
        if (st[i] != 2u) continue;
        if (!merge_entry(L, sm, cl, S, i)) spill_entry(L, sm, cl, S, i, sl);
    }
}

// merges spilled cache entries (after the table has been grown)
__global__ void merge_spilled_kernel(const __grid_constant__ VgAggLaunch L, int64_t n) {
    __shared__ Lay sl;
    if (threadIdx.x == 0) make_lay(L, (uint64_t)L.spill_cache_cap, sl);
    __syncthreads();
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        if (!merge_entry(L, L.spill_cache, sl, L.spill_cache_cap, i)) atomicOr(L.gt.err, VG_ERR_FULL);
}

// moves every occupied slot of `from` into the empty table `to`
struct RehashArgs {
    VgGroupTable from, to;
    int n_keys, n_accs;
    int32_t key_types[VG_MAX_KEYS];
    int32_t cls[VG_MAX_ACCS];
};

__global__ void rehash_kernel(const __grid_constant__ RehashArgs R) {
    const VgGroupTable &F = R.from, &T = R.to;
    KeyTypes kt;
#pragma unroll
    for (int j = 0; j < VG_MAX_KEYS; j++) kt.t[j] = R.key_types[j];
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < F.cap; i += stride) {
        if (F.state[i] != 2u) continue;
        Keys k;
#pragma unroll
        for (int j = 0; j < VG_MAX_KEYS; j++) k.w[j] = j < R.n_keys ? F.keys[(int64_t)j * F.cap + i] : 0;
        uint32_t nm = F.nullmask[i];
        int64_t g = gt_find_insert(T, k, R.n_keys, kt, nm, hash_k(k, R.n_keys, nm));
        if (g < 0) { atomicOr(T.err, VG_ERR_FULL); continue; }
        T.first_row[g] = F.first_row[i];
        for (int a = 0; a < R.n_accs; a++) {
            T.cnt[a][g] = F.cnt[a][i];
            T.flags[a][g] = F.flags[a][i];
            T.val[a][g] = F.val[a][i];
            if (R.cls[a] == VG_ACC_SUM_F64) {
                AccPtrs fp = global_ptrs(F, a), tp = global_ptrs(T, a);
                tp.base[g] = fp.base[i];
                for (int w = 0; w < kWin; w++) tp.win[(int64_t)w * T.cap + g] = fp.win[(int64_t)w * F.cap + i];
                tp.fs[g] = fp.fs[i];
                tp.fc[g] = fp.fc[i];
            }
        }
    }
}

// ---------------------------------------------------------------------
// table init / compact / finish
// ---------------------------------------------------------------------
__global__ void gt_init_kernel(VgGroupTable gt, int n_accs, const int32_t *cls_dev) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < gt.cap; i += stride) {
        gt.state[i] = 0;
        gt.nullmask[i] = 0;
        gt.first_row[i] = ~0ull;
        for (int a = 0; a < n_accs; a++) {
            int cls = cls_dev[a];
            gt.cnt[a][i] = 0;
            gt.flags[a][i] = 0;
            gt.val[a][i] = acc_is_min(cls) ? 0x7FFFFFFFFFFFFFFFll
                         : acc_is_max(cls) ? (int64_t)0x8000000000000000ull : 0;
            if (cls == VG_ACC_SUM_F64) {
                int64_t *l = gt.lacc[a];
                ((int32_t *)l)[i] = kBaseUnset;
                for (int w = 0; w < kWin; w++) l[gt.cap * (1 + w) + i] = 0;
                double *fs = (double *)(l + gt.cap * (1 + kWin));
                fs[i] = 0.0;
                fs[gt.cap + i] = 0.0;
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) { *gt.n_used = 0; *gt.err = 0; }
}

__global__ void compact_slots_kernel(const uint32_t *state, int64_t cap, int32_t *out, uint32_t *n) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    int64_t cap_pad = (cap + 31) & ~31ll;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap_pad; i += stride) {
        bool occ = i < cap && state[i] == 2u;
        uint32_t m = __ballot_sync(0xFFFFFFFFu, occ);
        uint32_t base = 0;
        if (lane == 0 && m) base = atomicAdd(n, (uint32_t)__popc(m));
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (occ) out[base + __popc(m & ((1u << lane) - 1))] = (int32_t)i;
    }
}

struct FinishArgs {
    VgGroupTable gt;
    int n_keys;
    int32_t key_types[VG_MAX_KEYS];
    int n_out;
    VgFinish fin[VG_MAX_OUTS];
    const int32_t *slots;
    int64_t n_groups;
    uint64_t *key_out[VG_MAX_KEYS];
    uint32_t *key_valid[VG_MAX_KEYS];
    double *out[VG_MAX_OUTS];
    uint32_t *out_valid[VG_MAX_OUTS];
    uint32_t *warn;
};

VG_DEV double sum_f64_result(const VgGroupTable &gt, int a, int64_t g, uint32_t flags) {
    AccPtrs p = global_ptrs(gt, a);
    int64_t w[VG_LACC_WORDS];
    for (int i = 0; i < VG_LACC_WORDS; i++) w[i] = 0;
    int b = p.base[g];
    if (b != kBaseUnset)
        for (int i = 0; i < kWin; i++) w[b + i] += p.win[(int64_t)i * gt.cap + g];
    double fb[2] = {p.fs[g], p.fc[g]};
    uint32_t special = flags & (4u | 8u | 16u);
    for (int j = 0; j < 2; j++) {
        VgDigits d = vg_split_double(vg_f64_to_bits(fb[j]));
        special |= d.special;
        if (d.lo >= 0) {
            w[d.lo] += d.d0;
            w[d.lo + 1] += d.d1;
            if (d.lo + 2 < VG_LACC_WORDS) w[d.lo + 2] += d.d2;
        }
    }
    return vg_digits_to_double(w, VG_LACC_WORDS, special);
}

__global__ void finish_kernel(const FinishArgs *__restrict__ F) {
    const int lane = threadIdx.x & 31;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t n_pad = (F->n_groups + 31) & ~31ll;
    const VgGroupTable &gt = F->gt;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n_pad; j += stride) {
        bool in = j < F->n_groups;
        int64_t g = in ? F->slots[j] : 0;
        uint32_t nm = in ? gt.nullmask[g] : 0xFFFFFFFFu;
        for (int k = 0; k < F->n_keys; k++) {
            bool ok = in && !((nm >> k) & 1u);
            if (in) F->key_out[k][j] = ok ? gt.keys[(int64_t)k * gt.cap + g] : 0;
            uint32_t m = __ballot_sync(0xFFFFFFFFu, ok);
            if (lane == 0) F->key_valid[k][j >> 5] = m;
        }
        for (int o = 0; o < F->n_out; o++) {
            const VgFinish &fi = F->fin[o];
            bool ok = false;
            double r = 0.0;
            if (in) {
                int a = fi.acc;
                uint64_t cnt = gt.cnt[a][g];
                uint32_t fl = gt.flags[a][g];
                int64_t v = gt.val[a][g];
                ok = true;
                switch (fi.finish) {
                case AGG_COUNT:
                case AGG_COUNT_STAR:
                    r = (double)cnt;   // exact below 2^53
                    break;
                case AGG_SUM:
                    if (fl & 1u) { ok = false; break; }
                    if (fi.in_type == VEC_DOUBLE) r = sum_f64_result(gt, a, g, fl);
                    else r = vg_i2f(v);
                    break;
                case AGG_MEAN:
                    if (fl & 1u) { ok = false; break; }
                    if (cnt == 0) { r = __longlong_as_double(0x7FF8000000000000ll); break; }
                    if (fi.in_type == VEC_DOUBLE) r = __ddiv_rn(sum_f64_result(gt, a, g, fl), (double)cnt);
                    else r = __ddiv_rn(vg_i2f(v), (double)cnt);
                    break;
                case AGG_MIN:
                case AGG_MAX: {
                    bool is_min = fi.finish == AGG_MIN;
                    if (fl & 1u) { ok = false; break; }
                    if (!(fl & 2u)) {
                        r = is_min ? __longlong_as_double(0x7FF0000000000000ll)
                                   : __longlong_as_double((long long)0xFFF0000000000000ull);
                        atomicAdd(F->warn, 1u);
                        break;
                    }
                    if (fl & 4u) { r = __longlong_as_double(0x7FF8000000000000ll); break; }
                    if (fi.in_type == VEC_DOUBLE) r = vg_bits_to_f64(vg_unord(v));
                    else r = vg_i2f(v);
                    break;
                }
                }
                F->out[o][j] = ok ? r : 0.0;
            }
            uint32_t m = __ballot_sync(0xFFFFFFFFu, in && ok);
            if (lane == 0) F->out_valid[o][j >> 5] = m;
        }
    }
}

// ---------------------------------------------------------------------
// ordering of the result groups
// ---------------------------------------------------------------------
// Sort key of a slot for key position k: NA last, then ascending value.
VG_DEV uint64_t order_word(const VgGroupTable &gt, int k, int type, int64_t g, bool &na) {
    na = (gt.nullmask[g] >> k) & 1u;
    uint64_t b = gt.keys[(int64_t)k * gt.cap + g];
    if (type == VEC_DOUBLE) return (uint64_t)vg_ord(b) ^ 0x8000000000000000ull;
    if (type == VEC_BOOL) return b;
    return b ^ 0x8000000000000000ull;
}

struct OrderArgs {
    VgGroupTable gt;
    int n_keys;
    int mode;
    int32_t key_types[VG_MAX_KEYS];
};

VG_DEV int cmp_slots(const OrderArgs &A, int32_t x, int32_t y) {
    if (A.mode == 1) {
        uint64_t a = A.gt.first_row[x], b = A.gt.first_row[y];
        return a < b ? -1 : a > b ? 1 : 0;
    }
    for (int k = 0; k < A.n_keys; k++) {
        bool na1, na2;
        uint64_t a = order_word(A.gt, k, A.key_types[k], x, na1);
        uint64_t b = order_word(A.gt, k, A.key_types[k], y, na2);
        if (na1 != na2) return na1 ? 1 : -1;
        if (na1) continue;
        if (a != b) return a < b ? -1 : 1;
    }
    return 0;
}

// one CTA: bitonic sort of up to 4096 slot ids in shared memory
__global__ void __launch_bounds__(1024) small_sort_kernel(OrderArgs A, int32_t *slots, int n) {
    __shared__ int32_t s[4096];
    int P = 1;
    while (P < n) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) s[i] = i < n ? slots[i] : -1;
    __syncthreads();
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                int j = i ^ stride;
                if (j > i) {
                    bool up = (i & size) == 0;
                    int32_t a = s[i], b = s[j];
                    // padding (-1) sorts after everything
                    int c = (a < 0) ? ((b < 0) ? 0 : 1) : (b < 0 ? -1 : cmp_slots(A, a, b));
                    if (c == 0) c = (a < b) ? -1 : (a > b ? 1 : 0);
                    if ((c > 0) == up) { s[i] = b; s[j] = a; }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) slots[i] = s[i];
}

__global__ void make_keys_kernel(OrderArgs A, const int32_t *slots, int64_t n, int key_idx,
                                 int na_pass, uint64_t *keys) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        int32_t g = slots[i];
        if (A.mode == 1) { keys[i] = A.gt.first_row[g]; continue; }
        bool na;
        uint64_t w = order_word(A.gt, key_idx, A.key_types[key_idx], g, na);
        keys[i] = na_pass ? (na ? 1u : 0u) : (na ? 0 : w);
    }
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

}  // namespace

extern "C" {

const char *vgk_agg_last_error(void) { return g_err; }

size_t vgk_agg_smem_bytes(const VgAggLaunch *L) {
    if (L->cache_slots <= 0) return 0;
    Lay c;
    make_lay(*L, (uint64_t)L->cache_slots, c);
    return c.total;
}

size_t vgk_agg_cache_bytes(const VgAggLaunch *L, int64_t slots) {
    Lay c;
    make_lay(*L, (uint64_t)slots, c);
    return c.total;
}

int vgk_group_table_init(VgGroupTable *gt, int n_keys, const int32_t *acc_cls, int n_accs,
                         vg_stream_t s) {
    (void)n_keys;
    cudaStream_t st = (cudaStream_t)s;
    int32_t *dcls = nullptr;
    if (check(cudaMallocAsync((void **)&dcls, 4 * (size_t)(n_accs > 0 ? n_accs : 1), st), "gt init")) return -1;
    cudaMemcpyAsync(dcls, acc_cls, 4 * (size_t)n_accs, cudaMemcpyHostToDevice, st);
    { gt_init_kernel<<<grid_for(gt->cap, 256), 256, 0, st>>>(*gt, n_accs, dcls); vg_launch_counter++; }
    cudaFreeAsync(dcls, st);
    return check(cudaGetLastError(), "gt init");
}

// bytes of the per-accumulator double-sum state in the global table
size_t vgk_lacc_bytes(int64_t cap) {
    return (size_t)cap * 8 * (1 + kWin) + (size_t)cap * 16;
}

int vgk_agg_launch(const VgAggLaunch *L, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    int64_t n_logical = L->replay ? L->replay_n : (L->sel ? L->sel_n : L->n_rows);
    if (n_logical <= 0) return 0;
    bool cache = L->cache_slots > 0 && !L->replay;
    size_t smem = cache ? vgk_agg_smem_bytes(L) : 0;
    bool pred = L->pred.n_terms > 0, join = L->has_join != 0;
    int sms = vgk_num_sms();
    int64_t want = (n_logical + kThreads - 1) / kThreads;
    int64_t cap = (int64_t)sms * (cache ? (smem <= 100 * 1024 ? 2 : 1) : 4);
    if (want > cap) want = cap;
    int grid = (int)(want < 1 ? 1 : want);
#define VG_LAUNCH(P, J, C)                                                              \
    do {                                                                                \
        auto k = agg_kernel<P, J, C>;                                                   \
        if (smem > 48 * 1024)                                                           \
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        k<<<grid, kThreads, smem, st>>>(*L, n_logical);                                  \
        vg_launch_counter++;                                                            \
    } while (0)
    vg_prof_begin(VG_PROF_AGG, st);
    if (pred) {
        if (join) { if (cache) VG_LAUNCH(true, true, true); else VG_LAUNCH(true, true, false); }
        else { if (cache) VG_LAUNCH(true, false, true); else VG_LAUNCH(true, false, false); }
    } else {
        if (join) { if (cache) VG_LAUNCH(false, true, true); else VG_LAUNCH(false, true, false); }
        else { if (cache) VG_LAUNCH(false, false, true); else VG_LAUNCH(false, false, false); }
    }
#undef VG_LAUNCH
    vg_prof_end(VG_PROF_AGG, st);
    return check(cudaGetLastError(), "agg launch");
}

int vgk_agg_merge_spilled_cache(const VgAggLaunch *L, int64_t n, vg_stream_t s) {
    if (n <= 0) return 0;
    cudaStream_t st = (cudaStream_t)s;
    merge_spilled_kernel<<<grid_for(n, 256), 256, 0, st>>>(*L, n);
    vg_launch_counter++;
    return check(cudaGetLastError(), "merge spilled");
}

int vgk_group_table_rehash(const VgGroupTable *from, const VgGroupTable *to, int n_keys,
                           const int32_t *key_types, const int32_t *acc_cls, int n_accs, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    RehashArgs R;
    memset(&R, 0, sizeof(R));
    R.from = *from;
    R.to = *to;
    R.n_keys = n_keys;
    R.n_accs = n_accs;
    for (int k = 0; k < n_keys; k++) R.key_types[k] = key_types[k];
    for (int a = 0; a < n_accs; a++) R.cls[a] = acc_cls[a];
    rehash_kernel<<<grid_for(from->cap, 256), 256, 0, st>>>(R);
    vg_launch_counter++;
    return check(cudaGetLastError(), "rehash");
}

int vgk_group_table_compact(const VgGroupTable *gt, int32_t *d_slots, uint32_t *h_n, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    uint32_t *dn = nullptr;
    if (check(cudaMallocAsync((void **)&dn, 4, st), "compact")) return -1;
    cudaMemsetAsync(dn, 0, 4, st);
    { compact_slots_kernel<<<grid_for(gt->cap, 256), 256, 0, st>>>(gt->state, gt->cap, d_slots, dn); vg_launch_counter++; }
    cudaMemcpyAsync(h_n, dn, 4, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(dn, st);
    return check(cudaStreamSynchronize(st), "compact");
}

int vgk_group_finish(const VgGroupTable *gt, int n_keys, const int32_t *key_types,
                     const int32_t *d_slots, int64_t n_groups, const VgFinish *fin, int n_out,
                     uint64_t **d_key_out, uint32_t **d_key_valid, double **d_out,
                     uint32_t **d_out_valid, uint32_t *d_warn, vg_stream_t s) {
    if (n_groups <= 0) return 0;
    if (n_out > VG_MAX_OUTS || n_keys > VG_MAX_KEYS) {
        snprintf(g_err, sizeof(g_err), "finish: too many outputs");
        return -1;
    }
    cudaStream_t st = (cudaStream_t)s;
    FinishArgs F;
    memset(&F, 0, sizeof(F));
    F.gt = *gt;
    F.n_keys = n_keys;
    for (int k = 0; k < n_keys; k++) {
        F.key_types[k] = key_types[k];
        F.key_out[k] = d_key_out[k];
        F.key_valid[k] = d_key_valid[k];
    }
    F.n_out = n_out;
    for (int o = 0; o < n_out; o++) {
        F.fin[o] = fin[o];
        F.out[o] = d_out[o];
        F.out_valid[o] = d_out_valid[o];
    }
    F.slots = d_slots;
    F.n_groups = n_groups;
    F.warn = d_warn;
    void *dF = nullptr;
    if (check(cudaMallocAsync(&dF, sizeof(F), st), "finish args")) return -1;
    cudaMemcpyAsync(dF, &F, sizeof(F), cudaMemcpyHostToDevice, st);
    vg_prof_begin(VG_PROF_FINISH, st);
    { finish_kernel<<<grid_for(n_groups, 128), 128, 0, st>>>((const FinishArgs *)dF); vg_launch_counter++; }
    vg_prof_end(VG_PROF_FINISH, st);
    cudaFreeAsync(dF, st);
    return check(cudaGetLastError(), "finish");
}

size_t vgk_order_scratch_bytes(int64_t n) {
    return a256((size_t)n * 8) + vgk_sort_pairs_scratch(n);
}

int vgk_order_groups(const VgGroupTable *gt, int n_keys, const int32_t *key_types, int32_t *d_slots,
                     int64_t n, int mode, void *d_scratch, size_t scratch_bytes, vg_stream_t s) {
    if (n <= 1) return 0;
    cudaStream_t st = (cudaStream_t)s;
    OrderArgs A;
    memset(&A, 0, sizeof(A));
    A.gt = *gt;
    A.n_keys = n_keys;
    A.mode = mode;
    for (int k = 0; k < n_keys; k++) A.key_types[k] = key_types[k];
    if (n <= 4096) {
        { small_sort_kernel<<<1, 1024, 0, st>>>(A, d_slots, (int)n); vg_launch_counter++; }
        return check(cudaGetLastError(), "small sort");
    }
    if (scratch_bytes < vgk_order_scratch_bytes(n)) {
        snprintf(g_err, sizeof(g_err), "order scratch too small");
        return -1;
    }
    uint64_t *keys = (uint64_t *)d_scratch;
    void *sort_scratch = (char *)d_scratch + a256((size_t)n * 8);
    size_t sort_bytes = scratch_bytes - a256((size_t)n * 8);
    // LSD over criteria: least significant key first; within a key, the
    // value passes come before the NA flag (NA sorts last)
    int n_crit = (mode == 1) ? 1 : n_keys;
    for (int c = n_crit - 1; c >= 0; c--) {
        for (int na_pass = 0; na_pass <= (mode == 1 ? 0 : 1); na_pass++) {
            { make_keys_kernel<<<grid_for(n, 256), 256, 0, st>>>(A, d_slots, n, c, na_pass, keys); vg_launch_counter++; }
            if (vgk_sort_pairs(keys, d_slots, n, na_pass ? 1 : 64, sort_scratch, sort_bytes, s)) {
                snprintf(g_err, sizeof(g_err), "%s", vgk_sort_last_error());
                return -1;
            }
        }
    }
    return check(cudaGetLastError(), "order");
}

}  // extern "C"
