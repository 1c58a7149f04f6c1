// k_groupby.cu -- grouped aggregation on sm_103a: the general fused kernel,
// spill / rehash kernels, result finishing and ordering.  The device helpers
// (exact fixed-point sums, shared-memory cache, global table) are in
// k_groupby_dev.cuh; the specialised kernel for common shapes is in
// k_groupby_fast.cu.

#include "k_groupby_dev.cuh"

extern "C" int vgk_agg_launch_fast(const VgAggLaunch *L, int64_t n_logical, vg_stream_t s);
extern "C" int vgk_agg_fast_ok(const VgAggLaunch *L);

namespace {

// ---------------------------------------------------------------------
// the fused aggregation kernel
// ---------------------------------------------------------------------
template <bool kCache>
__global__ void __launch_bounds__(kThreads, 2)
agg_kernel(const __grid_constant__ VgAggLaunch L, int64_t n_logical) {
    const bool kPred = L.pred.n_terms > 0;
    const bool kJoin = L.has_join != 0;
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
                            ((uint64_t)((li + L.li_base) & 0xFFFFFFFF) << 11) | rank;
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

// One output of group g (src/group_agg.c:240-281): counts, sums (NA if
// any input was NA and not removed), means, min / max (+-Inf with a
// warning for a group without values, as R's min/max).
VG_DEV double group_result(const VgGroupTable &gt, const VgFinish &fi, int64_t g, bool &ok, uint32_t *warn) {
    const int a = fi.acc;
    const uint64_t cnt = gt.cnt[a][g];
    const uint32_t fl = gt.flags[a][g];
    const int64_t v = gt.val[a][g];
    ok = true;
    switch (fi.finish) {
    case AGG_COUNT:
    case AGG_COUNT_STAR:
        return (double)cnt;   // exact below 2^53
    case AGG_SUM:
        if (fl & 1u) { ok = false; return 0.0; }
        if (fi.in_type == VEC_DOUBLE) return sum_f64_result(gt, a, g, fl);
        return vg_i2f(v);
    case AGG_MEAN:
        if (fl & 1u) { ok = false; return 0.0; }
        if (cnt == 0) return __longlong_as_double(0x7FF8000000000000ll);
        if (fi.in_type == VEC_DOUBLE) return __ddiv_rn(sum_f64_result(gt, a, g, fl), (double)cnt);
        return __ddiv_rn(vg_i2f(v), (double)cnt);
    default: {   // AGG_MIN, AGG_MAX
        const bool is_min = fi.finish == AGG_MIN;
        if (fl & 1u) { ok = false; return 0.0; }
        if (!(fl & 2u)) {
            atomicAdd(warn, 1u);
            return is_min ? __longlong_as_double(0x7FF0000000000000ll)
                          : __longlong_as_double((long long)0xFFF0000000000000ull);
        }
        if (fl & 4u) return __longlong_as_double(0x7FF8000000000000ll);
        if (fi.in_type == VEC_DOUBLE) return vg_bits_to_f64(vg_unord(v));
        return vg_i2f(v);
    }
    }
}

// The results of slot g written to one staging position (the NA-key
// group of the partitioned aggregation).
struct StageArgs {
    VgGroupTable gt;
    int n_out;
    VgFinish fin[VG_MAX_OUTS];
    int64_t slot;
    uint64_t pos;
    uint64_t *st_key;
    uint32_t *st_ok;
    double *st_out[VG_MAX_OUTS];
    uint32_t *warn;
};

__global__ void stage_kernel(const __grid_constant__ StageArgs A) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t okb = 0;
    for (int o = 0; o < A.n_out; o++) {
        bool ok = false;
        const double r = group_result(A.gt, A.fin[o], A.slot, ok, A.warn);
        A.st_out[o][A.pos] = ok ? r : 0.0;
        if (ok) okb |= 1u << o;
    }
    A.st_key[A.pos] = 0;
    A.st_ok[A.pos] = okb;
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
            bool ok = false;
            if (in) {
                const double r = group_result(gt, F->fin[o], g, ok, F->warn);
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

// One thread waits, through the table's own bounded wait, on a word that
// nothing will change; the expired wait is reported in the error word.
__global__ void wait_selftest_kernel(const uint32_t *busy_word, long long limit, uint32_t *err) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const uint32_t v = vg_wait_while(busy_word, 1u, vg_ld_acquire(busy_word), limit);
    if (v == 1u) atomicOr(err, VG_ERR_WAIT);
}

extern "C" {

// Runs wait_selftest_kernel: 0 and the error word read back in *code, or -1.
int vgk_wait_selftest(long long limit, uint32_t *code, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    uint32_t *d = nullptr;
    if (check(cudaMallocAsync((void **)&d, 256, st), "wait self-test")) return -1;
    uint32_t h[2] = {1u, 0u};
    if (check(cudaMemcpyAsync(d, h, 8, cudaMemcpyHostToDevice, st), "wait self-test")) return -1;
    wait_selftest_kernel<<<1, 32, 0, st>>>(d, limit, d + 1);
    vg_launch_counter++;
    cudaMemcpyAsync(h, d, 8, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (check(cudaStreamSynchronize(st), "wait self-test")) return -1;
    *code = h[1];
    return 0;
}

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
    int jrc = vgk_agg_launch_jit(L, n_logical, s);
    if (jrc == 1) return 0;
    if (jrc < 0) {
        snprintf(g_err, sizeof(g_err), "%s", vgk_jit_error());
        return -1;
    }
    if (vgk_agg_fast_ok(L)) return vgk_agg_launch_fast(L, n_logical, s);
    bool cache = L->cache_slots > 0 && !L->replay;
    size_t smem = cache ? vgk_agg_smem_bytes(L) : 0;
    int sms = vgk_num_sms();
    int64_t want = (n_logical + kThreads - 1) / kThreads;
    int64_t cap = (int64_t)sms * (cache ? (smem <= 100 * 1024 ? 2 : 1) : 4);
    if (want > cap) want = cap;
    int grid = (int)(want < 1 ? 1 : want);
#define VG_LAUNCH(C)                                                              \
    do {                                                                                \
        auto k = agg_kernel<C>;                                                   \
        if (smem > 48 * 1024)                                                           \
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        k<<<grid, kThreads, smem, st>>>(*L, n_logical);                                  \
        vg_launch_counter++;                                                            \
    } while (0)
    vg_prof_begin(VG_PROF_AGG, st);
    if (cache) VG_LAUNCH(true); else VG_LAUNCH(false);
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

int vgk_group_stage(const VgGroupTable *gt, const VgFinish *fin, int n_out, int64_t slot, uint64_t *st_key,
                    uint32_t *st_ok, double *const *st_out, uint64_t pos, uint32_t *d_warn, vg_stream_t s) {
    if (n_out > VG_MAX_OUTS) {
        snprintf(g_err, sizeof(g_err), "stage: too many outputs");
        return -1;
    }
    StageArgs A;
    memset(&A, 0, sizeof(A));
    A.gt = *gt;
    A.n_out = n_out;
    for (int o = 0; o < n_out; o++) {
        A.fin[o] = fin[o];
        A.st_out[o] = st_out[o];
    }
    A.slot = slot;
    A.pos = pos;
    A.st_key = st_key;
    A.st_ok = st_ok;
    A.warn = d_warn;
    { stage_kernel<<<1, 32, 0, (cudaStream_t)s>>>(A); vg_launch_counter++; }
    return check(cudaGetLastError(), "stage");
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
