// k_groupby_fast.cu -- the specialised form of the fused aggregation kernel.
//
// Taken for the common plan shapes: at most one group key, at most four
// accumulators, at most four probe columns (all 8-byte, 16-byte aligned), a
// dense batch (no selection vector) and, for joins, one key column.  It
// computes exactly what agg_kernel computes, in a layout tuned for the
// hardware:
//  * each thread owns 4 consecutive rows per step and issues every column
//    load for them (16-byte vector loads) before using any, so a warp keeps
//    ~4 KB of independent loads in flight;
//  * the 4 join probes are issued together, then the 4 build-row payloads;
//  * the accumulator count is a template parameter, so per-accumulator
//    shared-memory pointers live in registers;
//  * a group key with a small known range (a build-side attribute) indexes
//    the shared cache directly instead of hashing into it.
// Semantics are those of the reference's hash aggregation loop
// (hash_agg_next_batch, src/group_agg.c:155-281) with its accumulators
// (agg_accum_feed, src/agg_ops.c:93-158), behind a single-key join probe
// (join_probe_one, src/join.c:262-480) where the plan has one.

#include "k_groupby_dev.cuh"

namespace {

constexpr int kFastRows = 4;

// 4 validity bits of rows r..r+3 (r a multiple of 4) of a column
VG_DEV uint32_t valid4(const VgCol &c, int64_t r) {
    if (c.valid == nullptr) return 0xFu;
    int64_t b = r + c.voff;
    uint32_t w = __ldg(c.valid + (b >> 5));
    int s = (int)(b & 31);
    uint32_t bits = w >> s;
    if (s > 28) bits |= __ldg(c.valid + (b >> 5) + 1) << (32 - s);
    return bits & 0xFu;
}

struct Row4 {
    uint64_t v[4][kFastRows];   // [probe column][row]
    uint32_t ok[4];             // validity bits per probe column
};

VG_DEV void load_rows(const VgAggLaunch &L, int npc, int64_t r0, int64_t n, Row4 &R) {
    const bool full = r0 + kFastRows <= n;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        if (c >= npc) break;
        const VgCol &col = L.pcols[c];
        const unsigned long long *p = (const unsigned long long *)col.data + r0;
        if (full) {
            ulonglong2 a = __ldg((const ulonglong2 *)p);
            ulonglong2 b = __ldg((const ulonglong2 *)p + 1);
            R.v[c][0] = a.x; R.v[c][1] = a.y; R.v[c][2] = b.x; R.v[c][3] = b.y;
            R.ok[c] = valid4(col, r0);
        } else {
            uint32_t ok = 0;
#pragma unroll
            for (int j = 0; j < kFastRows; j++) {
                R.v[c][j] = 0;
                if (r0 + j < n) {
                    R.v[c][j] = __ldg(p + j);
                    if (vg_valid(col, r0 + j)) ok |= 1u << j;
                }
            }
            R.ok[c] = ok;
        }
    }
}

VG_DEV InVal operand4(const VgOperand &o, const Row4 &R, int j, const VgCol *bc, int64_t br) {
    InVal v;
    switch (o.side) {
    case VG_SIDE_PROBE:
        v.bits = R.v[o.col][j];
        v.ok = (R.ok[o.col] >> j) & 1u;
        return v;
    case VG_SIDE_BUILD:
        if (br < 0) { v.ok = false; v.bits = 0; return v; }
        v.ok = vg_valid(bc[o.col], br);
        v.bits = vg_load_bits(bc[o.col], br);
        return v;
    case VG_SIDE_LIT:
        v.ok = true; v.bits = (uint64_t)o.lit; return v;
    default:
        v.ok = false; v.bits = 0; return v;
    }
}

VG_DEV InVal value4(const VgValue &V, const Row4 &R, int j, const VgCol *bc, int64_t br) {
    InVal a = operand4(V.a, R, j, bc, br);
    if (V.op == 0) return a;
    InVal b = operand4(V.b, R, j, bc, br);
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
        case '*': z = __dmul_rn(x, y); break;
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

VG_DEV bool term4(const VgTerm &t, const Row4 &R, int j) {
    if (t.kind == VG_TERM_NONE) return false;
    bool v = (R.ok[t.col] >> j) & 1u;
    if (t.kind == VG_TERM_IS_NA) return !v;
    if (t.kind == VG_TERM_NOT_NA) return v;
    if (!v) return false;
    uint64_t bits = R.v[t.col][j];
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

// cache update with the count optionally skipped (no output reads it)
VG_DEV bool cache_update_fast(const VgAccSpec &A, const CPtrs &P, int64_t S, int64_t slot, InVal x, bool count) {
    const int cls = A.cls;
    if (cls == VG_ACC_COUNT_ALL) { atomicAdd(P.cnt + slot, 1u); return true; }
    if (cls == VG_ACC_COUNT_VALID) { if (x.ok) atomicAdd(P.cnt + slot, 1u); return true; }
    if (!x.ok) {
        if (!A.na_rm) set_flags(P.flags + slot, 1u);
        return true;
    }
    if (cls == VG_ACC_SUM_F64) {
        VgDigits d = vg_split_double(x.bits);
        if (d.special) set_flags(P.flags + slot, d.special);
        else if (d.lo >= 0 && !cwin_add(P.base + slot, P.wlo + slot, P.whi + slot, S, d)) return false;
        if (count) atomicAdd(P.cnt + slot, 1u);
        return true;
    }
    if (cls == VG_ACC_SUM_I64) {
        if (count) atomicAdd(P.cnt + slot, 1u);
        pair_add(P.vlo + slot, P.vhi + slot, (int64_t)x.bits);
        return true;
    }
    return cache_update(A, P, S, slot, x);
}

// NACC: accumulator slots compiled in (L.n_accs <= NACC)
template <int NACC, bool kPred, bool kJoin, bool kDense>
__global__ void __launch_bounds__(kThreads, 1)
agg_fast_kernel(const __grid_constant__ VgAggLaunch L, int64_t n_rows) {
    extern __shared__ __align__(16) char sm[];
    __shared__ Lay cl;
    __shared__ int cache_used;
    const int S = L.cache_slots;
    if (threadIdx.x == 0) { make_lay(L, S, cl); cache_used = 0; }
    __syncthreads();
    for (int i = threadIdx.x; i < S; i += blockDim.x) init_slot(L, sm, cl, S, i);
    if (kDense) {
        // keys are known: slot i holds dense_min + i, slot dense_n the NA key
        uint64_t *sk = (uint64_t *)(sm + cl.keys);
        uint32_t *snm = (uint32_t *)(sm + cl.nm);
        for (int i = threadIdx.x; i <= L.dense_n; i += blockDim.x) {
            sk[i] = i < L.dense_n ? (uint64_t)(L.dense_min + i) : 0;
            snm[i] = i < L.dense_n ? 0u : 1u;
        }
    }
    __syncthreads();
    const int nacc = L.n_accs;
    const KeyTypes kt = key_types(L);
    const int nk = L.n_keys;
    const int npc = L.n_pcols;
    uint32_t *st = (uint32_t *)(sm + cl.state);

    const int64_t tile = (int64_t)kFastRows * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * tile; base < n_rows; base += (int64_t)gridDim.x * tile) {
        const int64_t r0 = base + (int64_t)kFastRows * threadIdx.x;
        if (r0 >= n_rows) continue;
        Row4 R;
        load_rows(L, npc, r0, n_rows, R);
        uint32_t live = 0;
#pragma unroll
        for (int j = 0; j < kFastRows; j++) {
            bool keep = r0 + j < n_rows;
            if (kPred)
                for (int t = 0; t < L.pred.n_terms && keep; t++) keep = term4(L.pred.term[t], R, j);
            if (keep) live |= 1u << j;
        }
        // join: probe all 4 rows, first slots together
        int64_t brow[kFastRows];
        uint32_t matched = 0;
        if (kJoin) {
            uint64_t kw[kFastRows];
            int64_t slot[kFastRows];
            uint32_t need = 0;
            const int64_t mask = L.jt.cap - 1;
#pragma unroll
            for (int j = 0; j < kFastRows; j++) {
                brow[j] = -1;
                if (!((live >> j) & 1u)) continue;
                const int kc = L.jkey_col[0];
                if (!((R.ok[kc] >> j) & 1u)) continue;           // NA never matches
                uint64_t b = R.v[kc][j];
                if (L.jkey_conv[0]) b = vg_f64_to_bits(vg_i2f((int64_t)b));
                if (L.jt.key_types[0] == VEC_DOUBLE && vg_is_nan_bits(b)) continue;
                kw[j] = vg_norm_key(b, L.jt.key_types[0]);
                slot[j] = (int64_t)(vg_jhash(&kw[j], 1) & (uint64_t)mask);
                need |= 1u << j;
            }
            VgJSlot e[kFastRows];
#pragma unroll
            for (int j = 0; j < kFastRows; j++)
                if ((need >> j) & 1u) e[j] = jt_slot(L.jt.slots + (kw[j] == VG_JEMPTY ? L.jt.cap : slot[j]));
#pragma unroll
            for (int j = 0; j < kFastRows; j++) {
                if (!((need >> j) & 1u)) continue;
                if (kw[j] == VG_JEMPTY) {
                    if (e[j].count > 0) { brow[j] = e[j].start; matched |= 1u << j; }
                    continue;
                }
                int64_t s = slot[j];
                for (int64_t probe = 0; probe < L.jt.cap; probe++) {
                    if (e[j].key == kw[j]) { brow[j] = e[j].start; matched |= 1u << j; break; }
                    if (e[j].key == VG_JEMPTY) break;
                    s = (s + 1) & mask;
                    e[j] = jt_slot(L.jt.slots + s);
                }
            }
            if (L.join_kind != JOIN_LEFT) live &= matched;
        }
        // values and keys of the live rows, then the cache updates
#pragma unroll
        for (int j = 0; j < kFastRows; j++) {
            if (!((live >> j) & 1u)) continue;
            const int64_t br = kJoin ? brow[j] : -1;
            const int64_t li = r0 + j;
            uint64_t key = 0;
            uint32_t nm = 0;
            if (nk == 1) {
                InVal kv = value4(L.key[0], R, j, L.bcols, br);
                if (!kv.ok) nm = 1u;
                else key = vg_norm_key(kv.bits, kt.t[0]);
            }
            int found = -1;
            if (kDense) {
                found = nm ? L.dense_n : (int)((int64_t)key - L.dense_min);
                if (st[found] != 2u) st[found] = 2u;      // first touch marks the slot live
            } else {
                Keys k;
                k.w[0] = key; k.w[1] = 0; k.w[2] = 0; k.w[3] = 0;
                const uint64_t h = hash_k(k, nk, nm);
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
                            if (nk == 1) sk[slot] = key;
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
            uint64_t order = 0;
            if (L.track_first) {
                if (kJoin) {
                    bool m = (matched >> j) & 1u;
                    order = ((uint64_t)L.batch_idx << 44) | ((uint64_t)(m ? 0 : 1) << 43) |
                            ((uint64_t)((li + L.li_base) & 0xFFFFFFFF) << 11);
                } else {
                    order = (uint64_t)(L.row_base + li);
                }
            }
            if (found >= 0) {
                if (L.track_first)
                    atomicMin((unsigned long long *)(sm + cl.first) + found, (unsigned long long)order);
#pragma unroll
                for (int a = 0; a < NACC; a++) {
                    if (a >= nacc) break;
                    const VgAccSpec &A = L.acc[a];
                    InVal v = (A.cls == VG_ACC_COUNT_ALL) ? InVal{0, true} : value4(A.in, R, j, L.bcols, br);
                    if (cache_update_fast(A, cptrs(sm, cl, a, S), S, found, v, !((L.skip_count_mask >> a) & 1u)))
                        continue;
                    Keys k;
                    k.w[0] = key; k.w[1] = 0; k.w[2] = 0; k.w[3] = 0;
                    int64_t g = gt_find_insert(L.gt, k, nk, kt, nm, hash_k(k, nk, nm));
                    if (g >= 0) acc_update<true>(A, global_ptrs(L.gt, a), L.gt.cap, g, v);
                    else spill_row(L, li, 0, a);
                }
            } else {
                Keys k;
                k.w[0] = key; k.w[1] = 0; k.w[2] = 0; k.w[3] = 0;
                int64_t g = gt_find_insert(L.gt, k, nk, kt, nm, hash_k(k, nk, nm));
                if (g < 0) { spill_row(L, li, 0, -1); continue; }
                if (L.track_first) atomicMin((unsigned long long *)(L.gt.first_row + g), (unsigned long long)order);
#pragma unroll
                for (int a = 0; a < NACC; a++) {
                    if (a >= nacc) break;
                    const VgAccSpec &A = L.acc[a];
                    InVal v = (A.cls == VG_ACC_COUNT_ALL) ? InVal{0, true} : value4(A.in, R, j, L.bcols, br);
                    acc_update<true>(A, global_ptrs(L.gt, a), L.gt.cap, g, v);
                }
            }
        }
    }

    __syncthreads();
    __shared__ Lay sl;
    if (threadIdx.x == 0) make_lay(L, (uint64_t)L.spill_cache_cap, sl);
    __syncthreads();
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
        if (st[i] != 2u) continue;
        if (!merge_entry(L, sm, cl, S, i)) spill_entry(L, sm, cl, S, i, sl);
    }
}

}  // namespace

extern "C" {

#ifndef VG_FAST_PART
// The specialised kernel's preconditions.
int vgk_agg_fast_ok(const VgAggLaunch *L) {
    if (L->replay || L->sel || L->cache_slots <= 0) return 0;
    if (L->n_keys > 1 || L->n_accs > 4 || L->n_pcols > 4) return 0;
    for (int c = 0; c < L->n_pcols; c++) {
        if (L->pcols[c].type == VEC_BOOL) return 0;
        if (((uintptr_t)L->pcols[c].data) & 15) return 0;
    }
    if (L->has_join && (L->n_jkeys != 1 || !L->jt.slots || L->jt.rows || L->jt.direct)) return 0;
    if (L->dense && (L->n_keys != 1 || L->dense_n + 1 > L->cache_slots)) return 0;
    return 1;
}

int vgk_agg_launch_fast_join(const VgAggLaunch *L, int64_t n_logical, vg_stream_t s);
#endif

static int launch_fast(const VgAggLaunch *L, int64_t n_logical, vg_stream_t s, bool join) {
    cudaStream_t st = (cudaStream_t)s;
    Lay c;
    make_lay(*L, (uint64_t)L->cache_slots, c);
    size_t smem = c.total;
    int sms = vgk_num_sms();
    int64_t tiles = (n_logical + (int64_t)kFastRows * kThreads - 1) / ((int64_t)kFastRows * kThreads);
    int grid = (int)(tiles < sms ? (tiles < 1 ? 1 : tiles) : sms);
    const bool pred = L->pred.n_terms > 0;
    (void)join;
#define VG_FAST(P, J, D)                                                                     \
    do {                                                                                      \
        auto k = agg_fast_kernel<4, P, J, D>;                                                 \
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);      \
        k<<<grid, kThreads, smem, st>>>(*L, n_logical);                                       \
        vg_launch_counter++;                                                                  \
    } while (0)
    vg_prof_begin(VG_PROF_AGG, st);
#ifdef VG_FAST_PART
    if (L->dense) { if (pred) VG_FAST(true, true, true); else VG_FAST(false, true, true); }
    else { if (pred) VG_FAST(true, true, false); else VG_FAST(false, true, false); }
#else
    if (pred) VG_FAST(true, false, false); else VG_FAST(false, false, false);
#endif
#undef VG_FAST
    vg_prof_end(VG_PROF_AGG, st);
    return check(cudaGetLastError(), "agg launch (fast)");
}

#ifdef VG_FAST_PART
int vgk_agg_launch_fast_join(const VgAggLaunch *L, int64_t n_logical, vg_stream_t s) {
    return launch_fast(L, n_logical, s, true);
}
#else
int vgk_agg_launch_fast(const VgAggLaunch *L, int64_t n_logical, vg_stream_t s) {
    if (L->has_join) return vgk_agg_launch_fast_join(L, n_logical, s);
    return launch_fast(L, n_logical, s, false);
}
#endif

}  // extern "C"
