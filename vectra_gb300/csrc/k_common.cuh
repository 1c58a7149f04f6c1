// k_common.cuh -- device helpers shared by libvgpu's kernels (sm_103a).
// Validity follows the reference's bit-packed layout, bit i set = row i
// valid (VecArray.validity, src/types.h:47), read as 32-bit words.
#pragma once

#ifdef __CUDACC_RTC__
#include "vg_rtc_types.h"
#else
#include <cstdint>
#include <cuda_runtime.h>
#endif
#include "vgpu_internal.h"

#define VG_DEV __device__ __forceinline__

#ifndef __CUDACC_RTC__
// number of kernels this library has launched (reported by the benchmark)
extern "C" unsigned long long vg_launch_counter;

// optional event timing per kernel class (k_prof.cu); classes as in vgpu.h
#define VG_PROF_CLASSES 8
#define VG_PROF_AGG 0
#define VG_PROF_FILTER 1
#define VG_PROF_JOIN_BUILD 2
#define VG_PROF_JOIN_PROBE 3
#define VG_PROF_FINISH 4
#define VG_PROF_PAGG 5
void vg_prof_begin(int cls, cudaStream_t s);
void vg_prof_end(int cls, cudaStream_t s);
#endif

// ---------------------------------------------------------------------
// validity bits and column loads
// ---------------------------------------------------------------------

// Load with acquire semantics at device scope: the writes a releasing
// thread made before publishing this word are visible after it.
VG_DEV uint32_t vg_ld_acquire(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// 32-byte (256-bit) global store / streaming load of four 64-bit words;
// the address is 32-byte aligned (sm_100 family).
VG_DEV void vg_st256(void *p, uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
    asm volatile("st.global.v4.b64 [%0], {%1, %2, %3, %4};" ::"l"(p), "l"(a), "l"(b), "l"(c), "l"(d) : "memory");
}
VG_DEV void vg_ld256_cs(const void *p, uint64_t &a, uint64_t &b, uint64_t &c, uint64_t &d) {
    asm volatile("ld.global.cs.v4.b64 {%0, %1, %2, %3}, [%4];" : "=l"(a), "=l"(b), "=l"(c), "=l"(d) : "l"(p));
}

VG_DEV bool vg_valid(const VgCol &c, int64_t r) {
    r += c.voff;
    return c.valid == nullptr || ((__ldg(c.valid + (r >> 5)) >> (r & 31)) & 1u);
}

// 64-bit payload of a column value: int64 as is, double as its bit
// pattern, bool as 0/1.
VG_DEV uint64_t vg_load_bits(const VgCol &c, int64_t r) {
    if (c.type == VEC_BOOL) return (uint64_t)__ldg((const unsigned char *)c.data + r);
    return (uint64_t)__ldg((const unsigned long long *)c.data + r);
}

// the first four bytes of a string, big-endian, zero-padded
VG_DEV uint32_t vg_str_pre(const char *p, uint32_t len) {
    if (len == 0) return 0;
    const uint32_t last = len - 1;
    uint32_t pre = 0;
    for (uint32_t i = 0; i < 4; i++) {
        // read at a clamped position inside the string, then mask
        const uint32_t b = (uint32_t)(unsigned char)p[i < last ? i : last];
        pre = (pre << 8) | (i < len ? b : 0u);
    }
    return pre;
}

VG_DEV VgStrView vg_str_view(const char *p, uint32_t len) {
    VgStrView v;
    v.len = len;
    v.pre = vg_str_pre(p, len);
    v.ptr = p;
    return v;
}

VG_DEV double vg_bits_to_f64(uint64_t b) { return __longlong_as_double((long long)b); }
VG_DEV uint64_t vg_f64_to_bits(double d) { return (uint64_t)__double_as_longlong(d); }

// Order-preserving integer image of a double's bit pattern: for non-NaN x,y
// x < y  <=>  ord(x) < ord(y) (as signed int64), with -0 just below +0.
VG_DEV int64_t vg_ord(uint64_t bits) {
    int64_t s = (int64_t)bits;
    return s >= 0 ? s : (int64_t)(bits ^ 0x7FFFFFFFFFFFFFFFull);
}
VG_DEV uint64_t vg_unord(int64_t o) {
    return o >= 0 ? (uint64_t)o : ((uint64_t)o ^ 0x7FFFFFFFFFFFFFFFull);
}
VG_DEV bool vg_is_nan_bits(uint64_t b) {
    return (b & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull;
}

// Exact int64 -> double conversion with round-to-nearest-even (the C
// conversion the reference applies when it coerces int64 to double).
VG_DEV double vg_i2f(int64_t v) { return __ll2double_rn((long long)v); }

// ---------------------------------------------------------------------
// hashing (internal to the device tables; any good mixer will do since
// group / join membership depends only on key equality)
// ---------------------------------------------------------------------

VG_DEV uint64_t vg_mix64(uint64_t x) {
    // splitmix64 finaliser (Steele, Lea, Flood 2014)
    x ^= x >> 30; x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 27; x *= 0x94D049BB133111EBull;
    x ^= x >> 31;
    return x;
}

// Key words are normalised so that equal keys have equal words:
// doubles fold -0 onto +0.  NaN is kept as is; equality treats NaN as
// unequal to everything (double ==), handled by vg_key_word_eq.
VG_DEV uint64_t vg_norm_key(uint64_t bits, int type) {
    if (type == VEC_DOUBLE && bits == 0x8000000000000000ull) return 0;
    return bits;
}
VG_DEV bool vg_key_word_eq(uint64_t a, uint64_t b, int type) {
    if (type == VEC_DOUBLE && vg_is_nan_bits(a)) return false;
    return a == b;
}

VG_DEV uint64_t hash_keys(const uint64_t *k, int nk, uint32_t nm) {
    uint64_t h = 0x9E3779B97F4A7C15ull ^ nm;
    for (int i = 0; i < nk; i++) h = vg_mix64(h ^ k[i]) + (uint64_t)i;
    return vg_mix64(h);
}

// Slot hash of a join table key: one mixing round for the single-key
// tables (the common case, paid once per probe row), the general key hash
// for composite keys.
VG_DEV uint64_t vg_jhash(const uint64_t *k, int nk) {
    if (nk == 1) return vg_mix64(k[0] ^ 0x9E3779B97F4A7C15ull);
    return hash_keys(k, nk, 0);
}

// one 16-byte slot read through the read-only path
VG_DEV VgJSlot jt_slot(const VgJSlot *p) {
    ulonglong2 v = __ldg((const ulonglong2 *)p);
    VgJSlot s;
    s.key = v.x;
    s.start = (int32_t)(uint32_t)v.y;
    s.count = (int32_t)(uint32_t)(v.y >> 32);
    return s;
}

// Direct-addressed slot of key k, or -1 when k lies outside the table's range.
VG_DEV int64_t jt_direct_slot(const VgJoinTable &jt, uint64_t k) {
    const uint64_t d = k - (uint64_t)jt.dmin;
    return d < (uint64_t)jt.cap ? (int64_t)d : -1;
}

// Join table lookup: keys are normalised words of the common key types.
VG_DEV bool jt_lookup(const VgJoinTable &jt, const uint64_t *k, int32_t &start, int32_t &count) {
    if (jt.direct) {
        const int64_t d = jt_direct_slot(jt, k[0]);
        if (d < 0) return false;
        VgJSlot e = jt_slot(jt.slots + d);
        if (e.count <= 0) return false;
        start = e.start;
        count = e.count;
        return true;
    }
    uint64_t h = vg_jhash(k, jt.n_keys);
    const int64_t mask = jt.cap - 1;
    int64_t slot = (int64_t)(h & (uint64_t)mask);
    if (jt.slots) {
        if (k[0] == VG_JEMPTY) {
            VgJSlot e = jt_slot(jt.slots + jt.cap);
            if (e.count <= 0) return false;
            start = e.start;
            count = e.count;
            return true;
        }
        for (int64_t probe = 0; probe < jt.cap; probe++) {
            VgJSlot e = jt_slot(jt.slots + slot);
            if (e.key == k[0]) { start = e.start; count = e.count; return true; }
            if (e.key == VG_JEMPTY) return false;
            slot = (slot + 1) & mask;
        }
        return false;
    }
    for (int64_t probe = 0; probe < jt.cap; probe++) {
        uint32_t st = __ldg(jt.state + slot);
        if (st == 0) return false;
        bool eq = true;
        for (int i = 0; i < jt.n_keys && eq; i++)
            eq = __ldg((const unsigned long long *)jt.keys + (int64_t)i * jt.cap + slot) == k[i];
        if (eq) {
            start = __ldg(jt.start + slot);
            count = __ldg(jt.count + slot);
            return true;
        }
        slot = (slot + 1) & mask;
    }
    return false;
}

// build row of match m of a lookup (rows == NULL: unique keys, start is the row)
VG_DEV int64_t jt_row(const VgJoinTable &jt, int32_t start, int32_t m) {
    return jt.rows ? (int64_t)__ldg(jt.rows + start + m) : (int64_t)start;
}

// ---------------------------------------------------------------------
// exact double summation: fixed-point digit words
// ---------------------------------------------------------------------
//
// A finite double is m * 2^(sh-1074) with sh = max(E,1)-1 in [0, 2045] and
// m < 2^53.  In units of 2^-1074 it is m << sh, which spans at most three
// 32-bit digits starting at digit lo = sh/32.  Digits are accumulated as
// signed 64-bit words (32 bits of headroom each), so a group can take 2^31
// additions per word before any carry handling is needed; the finish
// step propagates carries and rounds once (round half to even).

struct VgDigits {
    int lo;            // first digit index, -1 for zero / non-finite
    int64_t d0, d1, d2; // signed digit contributions
    uint32_t special;  // bit2 NaN, bit3 +inf, bit4 -inf
};

__host__ __device__ inline VgDigits vg_split_double(uint64_t bits) {
    VgDigits r;
    uint32_t e = (uint32_t)((bits >> 52) & 0x7FF);
    uint64_t f = bits & 0x000FFFFFFFFFFFFFull;
    bool neg = (bits >> 63) != 0;
    r.special = 0;
    r.d0 = r.d1 = r.d2 = 0;
    if (e == 0x7FF) {
        r.lo = -1;
        r.special = f ? 4u : (neg ? 16u : 8u);
        return r;
    }
    uint64_t m = e ? (f | (1ull << 52)) : f;
    if (m == 0) { r.lo = -1; return r; }
    uint32_t sh = e ? e - 1 : 0;
    uint32_t off = sh & 31;
    r.lo = (int)(sh >> 5);
    uint64_t low = m << off;
    uint64_t high = off > 11 ? (m >> (64 - off)) : 0;
    int64_t a0 = (int64_t)(low & 0xFFFFFFFFull);
    int64_t a1 = (int64_t)(low >> 32);
    int64_t a2 = (int64_t)high;
    if (neg) { a0 = -a0; a1 = -a1; a2 = -a2; }
    r.d0 = a0; r.d1 = a1; r.d2 = a2;
    return r;
}

// The same split in 32-bit arithmetic, as magnitudes and a sign: the
// digits of |x| are d0, d1, d2 (unsigned) at digit index `word`.  zero:
// x is +-0 (nothing to add); special: as in VgDigits.
struct VgDigits32 {
    int word;
    uint32_t d0, d1, d2;
    uint32_t neg;
    uint32_t special;
    uint32_t zero;
};

// High word of (hi:lo) << s, s in [0, 31] (a funnel shift on the device).
__host__ __device__ inline uint32_t vg_fshl32(uint32_t lo, uint32_t hi, uint32_t s) {
#ifdef __CUDA_ARCH__
    return __funnelshift_l(lo, hi, s);
#else
    return s ? (hi << s) | (lo >> (32 - s)) : hi;
#endif
}

// Straight-line apart from the special case: the digits of a zero come out
// as 0 at word 0 (and zero is set).
__host__ __device__ inline VgDigits32 vg_split_double32(uint64_t bits) {
    VgDigits32 r;
    const uint32_t hi = (uint32_t)(bits >> 32), lo = (uint32_t)bits;
    const uint32_t e = (hi >> 20) & 0x7FFu;
    const uint32_t fh = hi & 0xFFFFFu;
    r.neg = hi >> 31;
    r.special = 0;
    if (e == 0x7FFu) {
        r.special = (fh | lo) ? 4u : (r.neg ? 16u : 8u);
        r.zero = 0;
        r.word = 0;
        r.d0 = r.d1 = r.d2 = 0;
        return r;
    }
    const uint32_t nz = e != 0u;
    const uint32_t mh = fh | (nz << 20);
    r.zero = (mh | lo) == 0u;
    const uint32_t sh = e - nz;            // subnormals share the exponent of the smallest normals
    const uint32_t off = sh & 31u;
    r.word = (int)(sh >> 5);
    // (mh:lo) << off spread over three 32-bit digits
    r.d0 = lo << off;
    r.d1 = vg_fshl32(lo, mh, off);
    r.d2 = vg_fshl32(mh, 0u, off);
    return r;
}

// Round the digit words (value = sum w[i] * 2^(32 i) units of 2^-1074,
// n words) to the nearest double, ties to even.
VG_DEV double vg_digits_to_double(const int64_t *w, int n, uint32_t special) {
    if (special & 4u) return __longlong_as_double(0x7FF8000000000000ll);
    if ((special & 8u) && (special & 16u)) return __longlong_as_double(0x7FF8000000000000ll);
    if (special & 8u) return __longlong_as_double(0x7FF0000000000000ll);
    if (special & 16u) return __longlong_as_double((long long)0xFFF0000000000000ull);
    // propagate carries into 32-bit digits
    uint32_t dig[VG_LACC_WORDS + 2];
    int64_t carry = 0;
    for (int i = 0; i < n; i++) {
        int64_t v = w[i] + carry;
        dig[i] = (uint32_t)(v & 0xFFFFFFFFll);
        carry = v >> 32;          // arithmetic shift
    }
    // remaining carry: sign-extend into two more digits
    dig[n] = (uint32_t)(carry & 0xFFFFFFFFll);
    dig[n + 1] = (uint32_t)((carry >> 32) & 0xFFFFFFFFll);
    int nd = n + 2;
    bool neg = carry < 0;
    if (neg) {   // two's complement negate
        uint64_t c = 1;
        for (int i = 0; i < nd; i++) {
            uint64_t v = (uint64_t)(uint32_t)~dig[i] + c;
            dig[i] = (uint32_t)v;
            c = v >> 32;
        }
    }
    int top = nd - 1;
    while (top >= 0 && dig[top] == 0) top--;
    if (top < 0) return 0.0;
    int lz = __clz(dig[top]);
    int p = top * 32 + (31 - lz);      // index of the leading one bit
    if (p >= 2098 + 64) {              // far beyond the double range
        return __longlong_as_double((long long)((neg ? 0xFFF0000000000000ull : 0x7FF0000000000000ull)));
    }
    uint64_t mant;
    int exp_field;
    if (p <= 52) {
        // exact: M < 2^53 units of 2^-1074
        uint64_t M = (uint64_t)dig[0] | ((top >= 1 ? (uint64_t)dig[1] : 0) << 32);
        if (M < (1ull << 52)) { mant = M; exp_field = 0; }
        else { mant = M & ((1ull << 52) - 1); exp_field = 1; }
    } else {
        // gather the 64 bits below and including bit p into `hi`
        int s = p - 63;                // bit index of hi's lsb (may be negative)
        uint64_t hi = 0;
        bool sticky = false;
        for (int i = 0; i < nd; i++) {
            int b0 = i * 32;           // digit i covers bits [b0, b0+32)
            if (b0 + 32 <= s) { if (dig[i]) sticky = true; continue; }
            if (b0 > p) break;
            uint64_t d = dig[i];
            int shift = b0 - s;        // position of digit's lsb within hi
            if (shift >= 0) hi |= d << shift;
            else {
                hi |= d >> (-shift);
                if (d & ((1ull << (-shift)) - 1)) sticky = true;
            }
        }
        // hi has the leading one at bit 63: keep 53 bits, round on the rest
        uint64_t keep = hi >> 11;
        uint64_t rest = hi & 0x7FF;
        bool round_bit = (rest >> 10) & 1;
        bool rest_sticky = sticky || (rest & 0x3FF);
        if (round_bit && (rest_sticky || (keep & 1))) keep++;
        int pp = p;
        if (keep >> 53) { keep >>= 1; pp++; }
        exp_field = pp - 51;
        if (exp_field >= 2047)
            return __longlong_as_double((long long)((neg ? 0xFFF0000000000000ull : 0x7FF0000000000000ull)));
        mant = keep & ((1ull << 52) - 1);
    }
    uint64_t bits = ((uint64_t)exp_field << 52) | mant;
    if (neg) bits |= 0x8000000000000000ull;
    return __longlong_as_double((long long)bits);
}

// The double nearest (ties to even) to six digit words w[0..6) at digit
// index base (value = sum w[i] 2^(32 (base + i)) units of 2^-1074, no
// special values): vg_digits_to_double's arithmetic on registers only, for
// kernels whose shared memory leaves little L1 for a thread-local array.
VG_DEV double vg_window6_to_double(const int64_t (&w)[6], int base) {
    constexpr int kWin = 6;
    uint32_t dig[kWin + 2];
    int64_t carry = 0;
#pragma unroll
    for (int i = 0; i < kWin; i++) {
        const int64_t v = w[i] + carry;
        dig[i] = (uint32_t)(v & 0xFFFFFFFFll);
        carry = v >> 32;
    }
    dig[kWin] = (uint32_t)(carry & 0xFFFFFFFFll);
    dig[kWin + 1] = (uint32_t)((carry >> 32) & 0xFFFFFFFFll);
    const bool neg = carry < 0;
    if (neg) {
        uint64_t c = 1;
#pragma unroll
        for (int i = 0; i < kWin + 2; i++) {
            const uint64_t v = (uint64_t)(uint32_t)~dig[i] + c;
            dig[i] = (uint32_t)v;
            c = v >> 32;
        }
    }
    uint64_t q[4];
#pragma unroll
    for (int j = 0; j < 4; j++) q[j] = (uint64_t)dig[2 * j] | ((uint64_t)dig[2 * j + 1] << 32);
    int top = -1;
#pragma unroll
    for (int j = 0; j < 4; j++)
        if (q[j]) top = j;
    if (top < 0) return 0.0;
    uint64_t qt = 0, q1 = 0;
    bool sticky = false;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        if (j == top) qt = q[j];
        if (j == top - 1) q1 = q[j];
        if (j < top - 1 && q[j]) sticky = true;
    }
    const int lz = __clzll((long long)qt);
    const int p = base * 32 + top * 64 + (63 - lz);     // index of the leading one bit
    const uint64_t inf = neg ? 0xFFF0000000000000ull : 0x7FF0000000000000ull;
    if (p >= 2098 + 64) return __longlong_as_double((long long)inf);
    uint64_t mant;
    int exp_field;
    if (p <= 52) {
        // exact: fewer than 2^53 units of 2^-1074 (then base <= 1 and top == 0)
        const uint64_t M = q[0] << (32 * base);
        if (M < (1ull << 52)) { mant = M; exp_field = 0; }
        else { mant = M & ((1ull << 52) - 1); exp_field = 1; }
    } else {
        const uint64_t hi = lz ? (qt << lz) | (q1 >> (64 - lz)) : qt;
        if (lz ? (q1 << lz) != 0 : q1 != 0) sticky = true;
        uint64_t keep = hi >> 11;
        const uint64_t rest = hi & 0x7FF;
        const bool round_bit = (rest >> 10) & 1;
        const bool rest_sticky = sticky || (rest & 0x3FF);
        if (round_bit && (rest_sticky || (keep & 1))) keep++;
        int pp = p;
        if (keep >> 53) { keep >>= 1; pp++; }
        exp_field = pp - 51;
        if (exp_field >= 2047) return __longlong_as_double((long long)inf);
        mant = keep & ((1ull << 52) - 1);
    }
    uint64_t bits = ((uint64_t)exp_field << 52) | mant;
    if (neg) bits |= 0x8000000000000000ull;
    return __longlong_as_double((long long)bits);
}

// ---------------------------------------------------------------------
// bounded waits
// ---------------------------------------------------------------------

#define VG_SPIN_LIMIT (1 << 22)

// Waits while the word at w holds `busy` (a slot another thread is still
// filling), starting from the value `v` already read, for at most `limit`
// polls with a short sleep between them.  Returns the value that ended the
// wait, or `busy` when the limit ran out: the caller then records
// VG_ERR_WAIT in its launch's error word and gives up, so the host sees an
// error status instead of a kernel that never ends.
VG_DEV uint32_t vg_wait_while(const uint32_t *w, uint32_t busy, uint32_t v, long long limit) {
    long long spins = 0;
    while (v == busy) {
        if (++spins > limit) return busy;
        __nanosleep(32);
        v = vg_ld_acquire(w);
    }
    return v;
}



