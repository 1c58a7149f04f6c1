// k_jit_lib.cuh -- device building blocks of the run-time specialised fused
// aggregation kernel (compiled by NVRTC together with the plan-specific
// definitions that jit_agg.cu generates, then k_jit_kernel.cuh).
//
// The generated part fixes at compile time everything the general kernel
// decides per row: which columns are read and their types, the predicate's
// term shapes, the join key, every group key and aggregate input
// expression, every accumulator's class and the shared-memory layout.  What
// stays a run-time value (column pointers, predicate bounds, table
// pointers, the dense key range) is read from the launch description in
// the constant bank.  Semantics are those of agg_kernel (k_groupby.cu),
// which in turn follow src/group_agg.c:155-281, src/agg_ops.c:93-158 and
// src/scalar_ops.c:11-66.
//
// Needs, defined before inclusion: VGJ_NPC, VGJ_NBC (probe / build columns
// read), VGJ_R (rows per thread).

#pragma once
#include "k_groupby_dev.cuh"

namespace vgj {

constexpr int R = VGJ_R;
constexpr int kNP = VGJ_NPC > 0 ? VGJ_NPC : 1;
constexpr int kNB = VGJ_NBC > 0 ? VGJ_NBC : 1;

// The rows one thread works on: values (raw 64-bit patterns) and validity
// bits of the probe columns and, after the join, of the build columns.
struct Rows {
    uint64_t p[kNP][R];
    uint32_t pok[kNP];
    uint64_t b[kNB][R];
    uint32_t bok[kNB];
};

// R validity bits of rows r..r+R-1 (r + voff aligned to R).
VG_DEV uint32_t valid_bits(const VgCol &c, int64_t r) {
    if (c.valid == nullptr) return (1u << R) - 1u;
    const int64_t b = r + c.voff;
    const uint32_t w = __ldg(c.valid + (b >> 5));
    return (w >> (int)(b & 31)) & ((1u << R) - 1u);
}

// Loads rows r0..r0+nv-1 of a probe column.  vec: r0 + R <= rows and the
// column's data and validity offsets allow whole vector loads.
template <int TYPE>
VG_DEV void load_dense(const VgCol &c, int64_t r0, int nv, bool vec, uint64_t (&v)[R], uint32_t &ok) {
    if (TYPE == VEC_BOOL) {
        const unsigned char *d = (const unsigned char *)c.data + r0;
        if (vec && R == 4) {
            uint32_t w = __ldg((const unsigned int *)d);
#pragma unroll
            for (int j = 0; j < R; j++) v[j] = (w >> (8 * j)) & 0xFFu;
        } else {
#pragma unroll
            for (int j = 0; j < R; j++) v[j] = j < nv ? (uint64_t)__ldg(d + j) : 0;
        }
    } else {
        const unsigned long long *d = (const unsigned long long *)c.data + r0;
        if (vec) {
#pragma unroll
            for (int j = 0; j < R; j += 2) {
                ulonglong2 a = __ldg((const ulonglong2 *)(d + j));
                v[j] = a.x;
                v[j + 1] = a.y;
            }
        } else {
#pragma unroll
            for (int j = 0; j < R; j++) v[j] = j < nv ? (uint64_t)__ldg(d + j) : 0;
        }
    }
    if (vec && ((r0 + c.voff) & (R - 1)) == 0) {
        ok = valid_bits(c, r0);
    } else {
        uint32_t m = 0;
#pragma unroll
        for (int j = 0; j < R; j++)
            if (j < nv && vg_valid(c, r0 + j)) m |= 1u << j;
        ok = m;
    }
}

// Loads the rows phys[0..nv) of a column (selection vector or build rows;
// entries < 0 are absent and read as NA).
template <int TYPE>
VG_DEV void load_rows(const VgCol &c, const int64_t (&phys)[R], uint32_t want, uint64_t (&v)[R], uint32_t &ok) {
    uint32_t m = 0;
#pragma unroll
    for (int j = 0; j < R; j++) {
        v[j] = 0;
        if (!((want >> j) & 1u)) continue;
        const int64_t r = phys[j];
        if (TYPE == VEC_BOOL) v[j] = (uint64_t)__ldg((const unsigned char *)c.data + r);
        else v[j] = (uint64_t)__ldg((const unsigned long long *)c.data + r);
        if (vg_valid(c, r)) m |= 1u << j;
    }
    ok = m;
}

// value = a op b in result type T (src/scalar_ops.c:11-66): operands
// coerced to T first; int64 division / modulo by zero is NA.
template <int OP, int T, int TA, int TB>
VG_DEV InVal arith(InVal a, InVal b) {
    InVal r;
    r.ok = a.ok && b.ok;
    r.bits = 0;
    if (!r.ok) return r;
    if (T == VEC_DOUBLE) {
        const double x = vg_bits_to_f64(TA == VEC_DOUBLE ? a.bits : vg_f64_to_bits(vg_i2f((int64_t)a.bits)));
        const double y = vg_bits_to_f64(TB == VEC_DOUBLE ? b.bits : vg_f64_to_bits(vg_i2f((int64_t)b.bits)));
        double z;
        if (OP == '+') z = __dadd_rn(x, y);
        else if (OP == '-') z = __dsub_rn(x, y);
        else if (OP == '*') z = __dmul_rn(x, y);   // one rounding, never fused
        else if (OP == '/') z = __ddiv_rn(x, y);
        else z = fmod(x, y);
        r.bits = vg_f64_to_bits(z);
    } else {
        const int64_t x = (int64_t)a.bits, y = (int64_t)b.bits;
        const uint64_t ux = (uint64_t)x, uy = (uint64_t)y;
        if (OP == '+') r.bits = ux + uy;
        else if (OP == '-') r.bits = ux - uy;
        else if (OP == '*') r.bits = ux * uy;
        else if (OP == '/') {
            if (y == 0) r.ok = false;
            else r.bits = (y == -1) ? (0 - ux) : (uint64_t)(x / y);
        } else {
            if (y == 0) r.ok = false;
            else r.bits = (y == -1) ? 0 : (uint64_t)(x % y);
        }
    }
    return r;
}

// Keep mask of the R rows for predicate term T (kind, column and domain
// fixed; bounds read from the launch description).
template <int KIND, int COL, int DOM, int NAN_KEEP, int T>
VG_DEV uint32_t term_mask(const VgAggLaunch &L, const Rows &X) {
    uint32_t m = 0;
    const uint32_t ok = X.pok[COL];
#pragma unroll
    for (int j = 0; j < R; j++) {
        const bool v = (ok >> j) & 1u;
        bool keep;
        if (KIND == VG_TERM_NONE) keep = false;
        else if (KIND == VG_TERM_IS_NA) keep = !v;
        else if (KIND == VG_TERM_NOT_NA) keep = v;
        else if (!v) keep = false;
        else {
            const uint64_t bits = X.p[COL][j];
            int64_t x;
            bool nan = false;
            if (DOM == VG_DOM_DOUBLE) {
                nan = vg_is_nan_bits(bits);
                x = vg_ord(bits);
            } else {
                x = (int64_t)bits;
            }
            if (nan) keep = NAN_KEEP != 0;
            else {
                const bool in = (x >= L.pred.term[T].lo) && (x <= L.pred.term[T].hi);
                keep = KIND == VG_TERM_RANGE ? in : !in;
            }
        }
        if (keep) m |= 1u << j;
    }
    return m;
}

// A double into a cache slot's digit window (same representation as
// cwin_add, in 32-bit arithmetic): each digit, negated for a negative
// summand, is added to the low word of its (lo, hi) pair as an unsigned
// 32-bit add; the high word then takes the add's carry, less one for a
// negated nonzero digit (so a borrow comes out as -1, no carry and no
// borrow as 0).  Written without branches apart from the rare ones (a
// special value, the slot's first value, a value outside the window): the
// adjustments are predicated atomics.  False: outside the window.
template <int S>
VG_DEV bool cache_sum_f64(char *sm, uint32_t OBASE, uint32_t OWIN, uint32_t *flags, int slot, uint64_t bits) {
    const VgDigits32 d = vg_split_double32(bits);
    if (d.special | d.zero) {
        if (d.special) set_flags(flags, d.special);
        return true;
    }
    int32_t *bp = (int32_t *)(sm + OBASE) + slot;
    int b = *(volatile int *)bp;
    if (b == kBaseUnset) {
        int want = d.word - 2;
        if (want < 0) want = 0;
        if (want > VG_LACC_WORDS - kWin) want = VG_LACC_WORDS - kWin;
        const int prev = atomicCAS((int *)bp, kBaseUnset, want);
        b = (prev == kBaseUnset) ? want : prev;
    }
    const int rel = d.word - b;
    // the value's digits take words rel .. rel+1 (+2 if d2 is nonzero)
    if ((unsigned)rel > (unsigned)(kWin - 2 - (d.d2 != 0u))) return false;
    uint32_t *wl = (uint32_t *)(sm + OWIN) + slot + rel * S;
    int32_t *wh = (int32_t *)(sm + OWIN + 4 * S * kWin) + slot + rel * S;
    const uint32_t m = 0u - d.neg;
    const uint32_t a0 = (d.d0 ^ m) + d.neg, a1 = (d.d1 ^ m) + d.neg, a2 = (d.d2 ^ m) + d.neg;
    const uint32_t o0 = atomicAdd(wl, a0);
    const uint32_t o1 = atomicAdd(wl + S, a1);
    uint32_t o2 = 0u;
    if (a2) o2 = atomicAdd(wl + 2 * S, a2);
    const int j0 = (int)(o0 + a0 < o0) - (int)(d.neg & (d.d0 != 0u));
    const int j1 = (int)(o1 + a1 < o1) - (int)(d.neg & (d.d1 != 0u));
    const int j2 = (int)(o2 + a2 < o2) - (int)(d.neg & (d.d2 != 0u));
    if (j0) atomicAdd(wh, j0);
    if (j1) atomicAdd(wh + S, j1);
    if (j2) atomicAdd(wh + 2 * S, j2);
    return true;
}

// The fused kernel's cache places every double sum of one accumulator on
// one digit window per CTA (not one per group): its base word is fixed by
// the first value the CTA adds (two words below it, as a group's own base
// would be) and held in a register by each thread, so a row's update reads
// no base from shared memory.  The kernel tail writes the CTA base into
// every live slot's base word before the slots are merged.  Values outside
// the window take the global table, as they do for a group's own window.
__shared__ int vgj_cta_base[VG_MAX_ACCS];

struct VgjBases {
    int b[VG_MAX_ACCS];
};

template <int S>
VG_DEV bool cache_sum_f64_cta(char *sm, uint32_t OWIN, uint32_t *flags, int slot, uint64_t bits, int &wb,
                              int *cta_base) {
    const VgDigits32 d = vg_split_double32(bits);
    if (d.special | d.zero) {
        if (d.special) set_flags(flags, d.special);
        return true;
    }
    if (wb == kBaseUnset) {
        int b = *(volatile int *)cta_base;
        if (b == kBaseUnset) {
            int want = d.word - 2;
            if (want < 0) want = 0;
            if (want > VG_LACC_WORDS - kWin) want = VG_LACC_WORDS - kWin;
            const int prev = atomicCAS(cta_base, kBaseUnset, want);
            b = (prev == kBaseUnset) ? want : prev;
        }
        wb = b;
    }
    const int rel = d.word - wb;
    if ((unsigned)rel > (unsigned)(kWin - 2 - (d.d2 != 0u))) return false;
    uint32_t *wl = (uint32_t *)(sm + OWIN) + slot + rel * S;
    int32_t *wh = (int32_t *)(sm + OWIN + 4 * S * kWin) + slot + rel * S;
    const uint32_t m = 0u - d.neg;
    const uint32_t a0 = (d.d0 ^ m) + d.neg, a1 = (d.d1 ^ m) + d.neg, a2 = (d.d2 ^ m) + d.neg;
    const uint32_t o0 = atomicAdd(wl, a0);
    const uint32_t o1 = atomicAdd(wl + S, a1);
    uint32_t o2 = 0u;
    if (a2) o2 = atomicAdd(wl + 2 * S, a2);
    const int j0 = (int)(o0 + a0 < o0) - (int)(d.neg & (d.d0 != 0u));
    const int j1 = (int)(o1 + a1 < o1) - (int)(d.neg & (d.d1 != 0u));
    const int j2 = (int)(o2 + a2 < o2) - (int)(d.neg & (d.d2 != 0u));
    if (j0) atomicAdd(wh, j0);
    if (j1) atomicAdd(wh + S, j1);
    if (j2) atomicAdd(wh + 2 * S, j2);
    return true;
}

// Accumulator update in the shared cache at compile-time layout offsets.
// False: the value falls outside the cache's digit window (the caller
// then updates the global table).
template <int CLS, int NA_RM, int COUNT, uint32_t OCNT, uint32_t OVAL, uint32_t OFLAGS, uint32_t OBASE,
          uint32_t OWIN, int S>
VG_DEV bool cache_acc(char *sm, int slot, InVal x) {
    uint32_t *cnt = (uint32_t *)(sm + OCNT) + slot;
    uint32_t *flags = (uint32_t *)(sm + OFLAGS) + slot;
    if (CLS == VG_ACC_COUNT_ALL) { atomicAdd(cnt, 1u); return true; }
    if (CLS == VG_ACC_COUNT_VALID) { if (x.ok) atomicAdd(cnt, 1u); return true; }
    if (!x.ok) {
        if (!NA_RM) set_flags(flags, 1u);
        return true;
    }
    if (CLS == VG_ACC_SUM_I64) {
        if (COUNT) atomicAdd(cnt, 1u);
        pair_add((uint32_t *)(sm + OVAL) + slot, (int32_t *)(sm + OVAL + 4 * S) + slot, (int64_t)x.bits);
        return true;
    }
    if (CLS == VG_ACC_SUM_F64) {
        if (!cache_sum_f64<S>(sm, OBASE, OWIN, flags, slot, x.bits)) return false;
        if (COUNT) atomicAdd(cnt, 1u);
        return true;
    }
    // 64-bit shared-memory min / max are compare-and-swap loops: only a
    // value that improves on the current one (which only moves one way)
    // takes the atomic
    long long *v64 = (long long *)(sm + OVAL) + slot;
    if (CLS == VG_ACC_MIN_I64 || CLS == VG_ACC_MAX_I64) {
        const long long v = (long long)x.bits, cur = *(volatile long long *)v64;
        if (CLS == VG_ACC_MIN_I64) { if (v < cur) atomicMin(v64, v); }
        else if (v > cur) atomicMax(v64, v);
        set_flags(flags, 2u);
        return true;
    }
    if (CLS == VG_ACC_MIN_F64 || CLS == VG_ACC_MAX_F64) {
        if (vg_is_nan_bits(x.bits)) { set_flags(flags, 2u | 4u); return true; }
        const long long v = (long long)vg_ord(x.bits), cur = *(volatile long long *)v64;
        if (CLS == VG_ACC_MIN_F64) { if (v < cur) atomicMin(v64, v); }
        else if (v > cur) atomicMax(v64, v);
        set_flags(flags, 2u);
        return true;
    }
    return true;   // VG_ACC_NA_ONLY
}

// cache_acc for the fused kernel's cache: double sums on the CTA's window
// (A = the accumulator's index), everything else as cache_acc.
template <int A, int CLS, int NA_RM, int COUNT, uint32_t OCNT, uint32_t OVAL, uint32_t OFLAGS, uint32_t OBASE,
          uint32_t OWIN, int S>
VG_DEV bool cache_acc_k(char *sm, int slot, InVal x, VgjBases &wb) {
    if (CLS != VG_ACC_SUM_F64) return cache_acc<CLS, NA_RM, COUNT, OCNT, OVAL, OFLAGS, OBASE, OWIN, S>(sm, slot, x);
    uint32_t *cnt = (uint32_t *)(sm + OCNT) + slot;
    uint32_t *flags = (uint32_t *)(sm + OFLAGS) + slot;
    if (!x.ok) {
        if (!NA_RM) set_flags(flags, 1u);
        return true;
    }
    if (!cache_sum_f64_cta<S>(sm, OWIN, flags, slot, x.bits, wb.b[A], &vgj_cta_base[A])) return false;
    if (COUNT) atomicAdd(cnt, 1u);
    return true;
}

// Finds or claims the cache slot of a key (open addressing, bounded
// probes; new keys only while the cache is under 3/4 full).  -1: not cached.
template <int S, int NK>
VG_DEV int cache_find(char *sm, uint32_t OSTATE, uint32_t ONM, uint32_t OKEYS, int *cache_used,
                      const Keys &k, uint32_t nm, const KeyTypes &kt, int *err) {
    uint32_t *st = (uint32_t *)(sm + OSTATE);
    uint32_t *snm = (uint32_t *)(sm + ONM);
    uint64_t *sk = (uint64_t *)(sm + OKEYS);
    const uint64_t h = hash_k(k, NK, nm);
    int slot = (int)(h & (uint64_t)(S - 1));
    const bool may_insert = *(volatile int *)cache_used < (S * 3) / 4;
    for (int probe = 0; probe < (may_insert ? kCacheProbes : 4); probe++) {
        uint32_t s0 = *(volatile uint32_t *)(st + slot);
        if (s0 == 0) {
            if (!may_insert) return -1;
            const uint32_t prev = atomicCAS(st + slot, 0u, 1u);
            if (prev == 0u) {
#pragma unroll
                for (int i = 0; i < NK; i++) sk[(int64_t)i * S + slot] = k.w[i];
                snm[slot] = nm;
                __threadfence_block();
                atomicExch(st + slot, 2u);
                atomicAdd(cache_used, 1);
                return slot;
            }
            s0 = prev;
        }
        int spins = 0;
        while (s0 == 1u) {
            if (++spins > VG_SPIN_LIMIT) { *err = 1; return -1; }
            s0 = *(volatile uint32_t *)(st + slot);
        }
        if (s0 != 2u) return -1;
        __threadfence_block();
        if (keys_eq(sk, S, slot, k, NK, kt, *(volatile uint32_t *)(snm + slot), nm)) return slot;
        slot = (slot + 1) & (S - 1);
    }
    return -1;
}

}  // namespace vgj
