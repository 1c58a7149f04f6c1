// k_jit_kernel.cuh -- the run-time specialised fused aggregation kernel.
//
// Included by the NVRTC source that jit_agg.cu generates for one plan,
// after k_jit_lib.cuh and the plan's hooks:
//   vgj_load_probe, vgj_pred, vgj_load_build, vgj_keys, vgj_cache_update,
//   vgj_global_update, vgj_spill
// and the VGJ_* constants.  One thread owns R consecutive logical rows per
// step: it issues every column load for them first, then the R join
// probes together, then the build-row loads, then the cache updates, so a
// warp keeps many independent memory requests in flight.  The CTA's groups
// live in a shared-memory cache (hashed, or dense when the group key is a
// build-side attribute with a small known range) and are merged into the
// global table when the CTA finishes; groups that do not fit in the cache,
// and digit-window overflows, update the global table directly; rows that
// find the global table full are spilled for a replay after it grows.
// Partition mode (VGJ_PART, hooks vgj_reserve / vgj_write): rows with a valid key are
// written as records into their key-range bucket instead; the cache then
// holds the NA-key group alone, one slot per warp.
// Semantics restated: hash_agg_next_batch (src/group_agg.c:155-281) with
// agg_accum_feed (src/agg_ops.c:93-158), behind join_probe_one
// (src/join.c:262-480; NA keys never match, src/join.c:77-113).
// Queued mode (VGJ_COMPACT: a filter, no join, no partition, no selection
// vector, no first-seen order): when few of a warp's rows pass the filter,
// their row numbers join a per-warp queue (one slot per lane) instead of
// being aggregated in place, where one or two live lanes would run the
// whole update path; a full queue is aggregated by all 32 lanes, each
// reloading its row.  A step in which more than 32 of the warp's rows pass
// is aggregated in place as usual.

#pragma once

// First-seen order code of logical row li (hash-path output order): probe
// batch, then matched rows before the batch's unmatched LEFT rows, then the
// row (join), or the row's stream position.
VG_DEV uint64_t vgj_order(const VgAggLaunch &L, int64_t li, uint32_t matched, int j) {
#if VGJ_JOIN
    return ((uint64_t)L.batch_idx << 44) | ((uint64_t)(((matched >> j) & 1u) ? 0 : 1) << 43) |
           ((uint64_t)((li + L.li_base) & 0xFFFFFFFF) << 11);
#else
    (void)matched;
    (void)j;
    return (uint64_t)(L.row_base + li);
#endif
}

#if VGJ_JOIN
// The join probe of the rows in `live` (R rows of X): their slot reads are
// issued together, then their payload entries (or build rows) are read.
// Returns the rows that matched; for an inner join, live loses the rest.
VG_DEV uint32_t vgj_join_probe(const VgAggLaunch &L, Rows &X, uint32_t &live) {
    uint32_t matched = 0;
    int64_t brow[R];
        {
            uint64_t kw[R];
            int64_t slot[R];
            uint32_t need = 0;
            const int64_t mask = L.jt.cap - 1;
#pragma unroll
            for (int j = 0; j < R; j++) {
                brow[j] = -1;
                kw[j] = 0;
                slot[j] = 0;
                if (!((live >> j) & 1u)) continue;
                if (!((X.pok[VGJ_JCOL] >> j) & 1u)) continue;           // NA never matches
                uint64_t b = X.p[VGJ_JCOL][j];
                if (VGJ_JCONV) b = vg_f64_to_bits(vg_i2f((int64_t)b));
                if (VGJ_JKT == VEC_DOUBLE && vg_is_nan_bits(b)) continue;
                kw[j] = vg_norm_key(b, VGJ_JKT);
#if VGJ_JDIRECT
                slot[j] = jt_direct_slot(L.jt, kw[j]);
                if (slot[j] < 0) continue;                           // outside the key range: no match
#else
                slot[j] = kw[j] == VG_JEMPTY ? L.jt.cap : (int64_t)(vg_jhash(&kw[j], 1) & (uint64_t)mask);
#endif
                need |= 1u << j;
            }
#if VGJ_PAY && VGJ_PAY16
            // compact payload copy of a direct table: one 16-byte entry per
            // probe, {kept column, narrowed column, validity}
            ulonglong2 ea[R];
#pragma unroll
            for (int j = 0; j < R; j++)
                if ((need >> j) & 1u) ea[j] = __ldg((const ulonglong2 *)L.jpay + slot[j]);
#pragma unroll
            for (int i = 0; i < kNB; i++) X.bok[i] = 0;
#pragma unroll
            for (int j = 0; j < R; j++) {
                if (!((need >> j) & 1u)) continue;
                const uint32_t meta = (uint32_t)(ea[j].y >> 32);
                if (!(meta & 1u)) continue;
                matched |= 1u << j;
                brow[j] = 0;
                if (VGJ_PAY_NARROW < 0) {
                    X.b[0][j] = ea[j].x;
                    X.bok[0] |= ((meta >> 1) & 1u) << j;
                } else {
                    constexpr int kN = VGJ_PAY_NARROW < 0 ? 0 : VGJ_PAY_NARROW;
                    constexpr int kK = kNB > 1 ? 1 - kN : 0;
                    const uint32_t b = (uint32_t)ea[j].y;
                    X.b[kK][j] = ea[j].x;
                    X.b[kN][j] = VGJ_PAY_NARROW_T == VEC_BOOL ? (uint64_t)b : (uint64_t)L.jpay_min + (uint64_t)b;
                    X.bok[0] |= ((meta >> 1) & 1u) << j;
                    if (kNB > 1) X.bok[kNB > 1 ? 1 : 0] |= ((meta >> 2) & 1u) << j;
                }
            }
#elif VGJ_PAY
            // payload copy: key, build row, validity and up to two build
            // columns in one 32-byte sector per probe
            ulonglong2 ea[R], eb[R];
#pragma unroll
            for (int j = 0; j < R; j++) {
                if (!((need >> j) & 1u)) continue;
                const VgJPay *q = L.jpay + slot[j];
                ea[j] = __ldg((const ulonglong2 *)q);
                eb[j] = __ldg((const ulonglong2 *)q + 1);
            }
#pragma unroll
            for (int i = 0; i < kNB; i++) X.bok[i] = 0;
#pragma unroll
            for (int j = 0; j < R; j++) {
                if (!((need >> j) & 1u)) continue;
                bool hit;
                if (VGJ_JDIRECT || kw[j] == VG_JEMPTY) {
                    hit = ((ea[j].y >> 32) & 1u) != 0;
                } else {
                    hit = false;
                    int64_t s = slot[j];
                    for (int64_t probe = 0; probe < L.jt.cap; probe++) {
                        if (ea[j].x == kw[j]) { hit = true; break; }
                        if (ea[j].x == VG_JEMPTY) break;
                        s = (s + 1) & mask;
                        const VgJPay *q = L.jpay + s;
                        ea[j] = __ldg((const ulonglong2 *)q);
                        eb[j] = __ldg((const ulonglong2 *)q + 1);
                    }
                }
                if (hit) {
                    const uint32_t meta = (uint32_t)(ea[j].y >> 32);
                    brow[j] = (int64_t)(int32_t)(uint32_t)ea[j].y;
                    matched |= 1u << j;
                    X.b[0][j] = eb[j].x;
                    X.bok[0] |= ((meta >> 1) & 1u) << j;
                    if (kNB > 1) {
                        X.b[kNB > 1 ? 1 : 0][j] = eb[j].y;
                        X.bok[kNB > 1 ? 1 : 0] |= ((meta >> 2) & 1u) << j;
                    }
                }
            }
#else
            VgJSlot e[R];
#pragma unroll
            for (int j = 0; j < R; j++)
                if ((need >> j) & 1u) e[j] = jt_slot(L.jt.slots + slot[j]);
#pragma unroll
            for (int j = 0; j < R; j++) {
                if (!((need >> j) & 1u)) continue;
                if (VGJ_JDIRECT || kw[j] == VG_JEMPTY) {
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
#endif
            (void)mask;
            if (VGJ_JKIND != JOIN_LEFT) live &= matched;
        }
#if !VGJ_PAY
        vgj_load_build(L, X, brow, live & matched);
#else
        (void)brow;
#endif
    return matched;
}
#endif

#if VGJ_DEFER
// Dense cache: a row whose double sums fell outside the CTA's digit window
// is marked (one bit per row and double-sum accumulator) instead of
// updating the global table in the row loop, so the loop carries no
// global-table code and keeps its registers; the replay kernel below,
// launched after this one, applies the marks.
VG_DEV void vgj_defer_row(const VgAggLaunch &L, int64_t li, uint32_t which) {
    uint32_t n = 0;
    int f = 0;
#pragma unroll
    for (int a = 0; a < VG_MAX_ACCS; a++) {
        if (!((VGJ_F64_MASK >> a) & 1u)) continue;
        if ((which >> a) & 1u) {
            atomicOr(L.defer_bits + (int64_t)f * L.defer_words + (li >> 5), 1u << (int)(li & 31));
            n++;
        }
        f++;
    }
    atomicAdd(L.defer_n, n);
}

// Applies and clears the marks of the launch before it (same plan, same
// rows): each marked row is read again from device memory and its marked
// accumulators update the global table.  Returns at once when there are
// none.
extern "C" __global__ void __launch_bounds__(256)
vg_jit_replay(const __grid_constant__ VgAggLaunch L, int64_t n_rows) {
    using namespace vgj;
    (void)n_rows;
    if (*(volatile const uint32_t *)L.defer_n == 0u) return;
    const KeyTypes kt = key_types(L);
    int f = 0;
#pragma unroll
    for (int a = 0; a < VG_MAX_ACCS; a++) {
        if (!((VGJ_F64_MASK >> a) & 1u)) continue;
        uint32_t *bits = L.defer_bits + (int64_t)f * L.defer_words;
        f++;
        for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < L.defer_words;
             w += (int64_t)gridDim.x * blockDim.x) {
            uint32_t m = bits[w];
            if (!m) continue;
            bits[w] = 0u;
            while (m) {
                const int b = __ffs(m) - 1;
                m &= m - 1u;
                const int64_t li = w * 32 + b;
                Rows X;
                int64_t phys[R];
#pragma unroll
                for (int j = 0; j < R; j++) phys[j] = 0;
#if VGJ_SEL
                phys[0] = (int64_t)__ldg(L.sel + li);
#else
                phys[0] = li;
#endif
                vgj_load_probe(L, X, li, 1, false, phys, 1u);
#if VGJ_JOIN
                uint32_t live = 1u;
                (void)vgj_join_probe(L, X, live);
#endif
                Keys k;
#pragma unroll
                for (int i = 0; i < VG_MAX_KEYS; i++) k.w[i] = 0;
                uint32_t nm = 0;
                vgj_keys(X, 0, k, nm);
                const int64_t g = gt_find_insert(L.gt, k, VGJ_NK, kt, nm, hash_k(k, VGJ_NK, nm));
                if (g < 0) vgj_spill(L, li, 1u << a);
                else vgj_global_update(L, g, X, 0, 1u << a);
            }
        }
    }
}
#endif

extern "C" __global__ void __launch_bounds__(VGJ_THREADS, VGJ_MINB)
vg_jit_agg(const __grid_constant__ VgAggLaunch L, int64_t n_rows) {
    using namespace vgj;
    extern __shared__ __align__(16) char sm[];
    __shared__ Lay cl;
    __shared__ int cache_used;
    constexpr int S = VGJ_S;
    if (threadIdx.x == 0) {
        make_lay(L, S, cl);
        cache_used = 0;
    }
    if (threadIdx.x < VG_MAX_ACCS) vgj_cta_base[threadIdx.x] = kBaseUnset;
    VgjBases wb;
#pragma unroll
    for (int a = 0; a < VG_MAX_ACCS; a++) wb.b[a] = kBaseUnset;
    __syncthreads();
    for (int i = threadIdx.x; i < S; i += blockDim.x) init_slot(L, sm, cl, S, i);
#if VGJ_DENSE
    {
        uint64_t *sk = (uint64_t *)(sm + VGJ_OFF_KEYS);
        uint32_t *snm = (uint32_t *)(sm + VGJ_OFF_NM);
        for (int i = threadIdx.x; i <= L.dense_n; i += blockDim.x) {
            sk[i] = i < L.dense_n ? (uint64_t)(L.dense_min + i) : 0;
            snm[i] = i < L.dense_n ? 0u : 1u;
        }
    }
#endif
#if VGJ_PART
    {
        // partition mode: the cache holds the NA-key group only, one slot per warp
        uint64_t *sk = (uint64_t *)(sm + VGJ_OFF_KEYS);
        uint32_t *snm = (uint32_t *)(sm + VGJ_OFF_NM);
        for (int i = threadIdx.x; i < S; i += blockDim.x) {
            sk[i] = 0;
            snm[i] = 1u;
        }
    }
#if VGJ_PART_CTA
    {
        // this CTA's next position in each bucket (the region holds fewer
        // than 2^32 records)
        uint32_t *pc = (uint32_t *)(sm + VGJ_OFF_PCUR);
        for (int i = threadIdx.x; i < L.po.n_buckets; i += blockDim.x)
            pc[i] = (uint32_t)L.po.cta_off[(int64_t)i * gridDim.x + blockIdx.x];
    }
#endif
#endif
    __syncthreads();
    uint32_t *st = (uint32_t *)(sm + VGJ_OFF_STATE);
    const KeyTypes kt = key_types(L);

    const int64_t tile = (int64_t)R * blockDim.x;
    const int64_t step = (int64_t)gridDim.x * tile;
#if VGJ_PIPE
    // software pipeline: the probe columns of a thread's next rows are
    // loaded before its current rows are processed
    Rows Xn;
    {
        const int64_t r0n = (int64_t)blockIdx.x * tile + (int64_t)R * threadIdx.x;
        if (r0n < n_rows) {
            const int nvn = (int)(n_rows - r0n < R ? n_rows - r0n : R);
            int64_t physn[R];
#pragma unroll
            for (int j = 0; j < R; j++) physn[j] = r0n + j;
            vgj_load_probe(L, Xn, r0n, nvn, VGJ_VEC && nvn == R, physn, (1u << nvn) - 1u);
        }
    }
#endif
#if VGJ_COMPACT
    // the warp's queue: lane i holds slot i, qn slots are used (warp-uniform)
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t qn = 0;
    int64_t qrow = 0;
    // aggregates the first nq queued rows, one per lane (the hashed-cache
    // update of the in-place path below, for one row)
    auto flush_queue = [&](uint32_t nq) {
        if (lane >= nq) return;
        Rows Q;
        int64_t qp[R];
#pragma unroll
        for (int j = 0; j < R; j++) qp[j] = qrow;
        vgj_load_probe(L, Q, qrow, 1, false, qp, 1u);
        Keys k;
#pragma unroll
        for (int i = 0; i < VG_MAX_KEYS; i++) k.w[i] = 0;
        uint32_t nm = 0;
        vgj_keys(Q, 0, k, nm);
        int err = 0;
        const int found =
            cache_find<S, VGJ_NK>(sm, VGJ_OFF_STATE, VGJ_OFF_NM, VGJ_OFF_KEYS, &cache_used, k, nm, kt, &err);
        if (err) atomicOr(L.gt.err, VG_ERR_WAIT);
        const uint32_t fail = found < 0 ? 0u : vgj_cache_update(sm, found, Q, 0, wb);
        if (found >= 0 && !fail) return;
        const int64_t g = gt_find_insert(L.gt, k, VGJ_NK, kt, nm, hash_k(k, VGJ_NK, nm));
        if (g < 0) {
            if (found < 0) spill_row(L, qrow, 0, -1);
            else vgj_spill(L, qrow, fail);
            return;
        }
        vgj_global_update(L, g, Q, 0, found < 0 ? 0xFFFFFFFFu : fail);
    };
#endif
    for (int64_t base = (int64_t)blockIdx.x * tile; base < n_rows; base += step) {
        const int64_t r0 = base + (int64_t)R * threadIdx.x;
#if VGJ_COMPACT
        // every lane takes every step (the queue below is warp-collective);
        // lanes past the end have no rows
        const bool in_range = r0 < n_rows;
#else
        if (r0 >= n_rows) continue;
        const bool in_range = true;
#endif
        const int nv = in_range ? (int)(n_rows - r0 < R ? n_rows - r0 : R) : 0;
        const uint32_t all = (1u << nv) - 1u;
        int64_t phys[R];
#pragma unroll
        for (int j = 0; j < R; j++) {
#if VGJ_SEL
            phys[j] = j < nv ? (int64_t)__ldg(L.sel + r0 + j) : 0;
#else
            phys[j] = r0 + j;
#endif
        }
        Rows X;
#if VGJ_PIPE
        X = Xn;
        {
            const int64_t r0n = r0 + step;
            if (r0n < n_rows) {
                const int nvn = (int)(n_rows - r0n < R ? n_rows - r0n : R);
                int64_t physn[R];
#pragma unroll
                for (int j = 0; j < R; j++) physn[j] = r0n + j;
                vgj_load_probe(L, Xn, r0n, nvn, VGJ_VEC && nvn == R, physn, (1u << nvn) - 1u);
            }
        }
#else
        vgj_load_probe(L, X, r0, nv, VGJ_VEC && nv == R, phys, all);
#endif
        uint32_t live = all;
#if VGJ_PRED
        live &= vgj_pred(L, X);
#endif
#if VGJ_COMPACT
        {
            // the step's passing rows, numbered across the warp in lane order
            const uint32_t cnt = (uint32_t)__popc(live);
            uint32_t incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= (uint32_t)o) incl += v;
            }
            const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
            if (total == 0u) continue;
            if (total <= 32u) {
                // slot s takes the step's row k = (s - qn) mod 32: slots
                // qn..31 first, then, after the queue is aggregated, the
                // slots from 0 on
                const uint32_t k = (lane - qn) & 31u;
                uint32_t pos = 0;                   // owner: the lanes whose rows end at or before k
#pragma unroll
                for (uint32_t w = 16; w; w >>= 1) {
                    const uint32_t v = __shfl_sync(0xFFFFFFFFu, incl, pos + w - 1);
                    if (v <= k) pos += w;
                }
                const uint32_t o_excl = __shfl_sync(0xFFFFFFFFu, incl - cnt, pos);
                const uint32_t o_live = __shfl_sync(0xFFFFFFFFu, live, pos);
                const int64_t o_r0 = __shfl_sync(0xFFFFFFFFu, r0, pos);
                const bool has = k < total;
                uint32_t m = o_live;                // the (k - o_excl)-th live row of the owner
                const uint32_t t = k - o_excl;
#pragma unroll
                for (uint32_t i = 0; i + 1 < (uint32_t)R; i++)
                    if (i < t) m &= m - 1u;
                const int64_t row = o_r0 + (int64_t)(__ffs(m) - 1);
                if (has && lane >= qn) qrow = row;
                if (qn + total >= 32u) {
                    flush_queue(32u);
                    const uint32_t before = qn;
                    qn = qn + total - 32u;
                    if (has && lane < before) qrow = row;
                } else {
                    qn += total;
                }
                continue;
            }
        }
#endif
        uint32_t matched = 0;
#if VGJ_JOIN
        matched = vgj_join_probe(L, X, live);
#endif
#if VGJ_PART
        // Partition mode: the rows with a valid key claim their record
        // positions first (all R cursor atomics in flight together), then
        // write their records; the NA-key rows stay live for the cache.
        {
            unsigned long long pos[R];
            uint64_t kk[R];
            uint32_t emit = 0;
#pragma unroll
            for (int j = 0; j < R; j++) {
                pos[j] = 0;
                kk[j] = 0;
                if (!((live >> j) & 1u)) continue;
                Keys k;
#pragma unroll
                for (int i = 0; i < VG_MAX_KEYS; i++) k.w[i] = 0;
                uint32_t nm = 0;
                vgj_keys(X, j, k, nm);
                if (nm) continue;
                kk[j] = k.w[0];
                pos[j] = vgj_reserve(L, sm, kk[j]);
                emit |= 1u << j;
            }
#pragma unroll
            for (int j = 0; j < R; j++)
                if ((emit >> j) & 1u) vgj_write(L, pos[j], kk[j], X, j);
            live &= ~emit;
        }
#endif
        // Cache updates.  Rows that need the global table (a hashed-cache
        // miss, or a value outside a cache digit window) are only marked
        // here and handled together afterwards, so the per-row path has no
        // rarely-taken branches around global atomics.
        uint32_t rare = 0, miss = 0;
        uint32_t failm[R];
#pragma unroll
        for (int j = 0; j < R; j++) {
            failm[j] = 0;
            if (!((live >> j) & 1u)) continue;
            Keys k;
#pragma unroll
            for (int i = 0; i < VG_MAX_KEYS; i++) k.w[i] = 0;
            uint32_t nm = 0;
            vgj_keys(X, j, k, nm);
            int found;
#if VGJ_PART
            (void)cache_used;
            found = (int)(threadIdx.x >> 5);             // an NA-key row: the warp's slot
            st[found] = 2u;
#elif VGJ_DENSE
            (void)cache_used;
            found = nm ? L.dense_n : (int)((int64_t)k.w[0] - L.dense_min);
#if !VGJ_LIVE_BY_CNT
            st[found] = 2u;                           // every touch marks the slot live (same value)
#endif
#else
            {
                int err = 0;
                found = cache_find<S, VGJ_NK>(sm, VGJ_OFF_STATE, VGJ_OFF_NM, VGJ_OFF_KEYS, &cache_used, k, nm,
                                              kt, &err);
                if (err) atomicOr(L.gt.err, VG_ERR_WAIT);
            }
            if (found < 0) {
                miss |= 1u << j;
                continue;
            }
#endif
#if VGJ_TRACK
            atomicMin((unsigned long long *)(sm + VGJ_OFF_FIRST) + found, (unsigned long long)vgj_order(L, r0 + j, matched, j));
#endif
            failm[j] = vgj_cache_update(sm, found, X, j, wb);
            if (failm[j]) rare |= 1u << j;
        }
#if VGJ_DEFER
        // rows for the global table are marked for the replay (a dense cache never misses)
        (void)miss;
        if (rare) {
#pragma unroll
            for (int j = 0; j < R; j++)
                if ((rare >> j) & 1u) vgj_defer_row(L, r0 + j, failm[j]);
        }
#else
        if (rare | miss) {
#pragma unroll
            for (int j = 0; j < R; j++) {
                const bool m = (miss >> j) & 1u;
                if (!m && !((rare >> j) & 1u)) continue;
                const int64_t li = r0 + j;
                Keys k;
#pragma unroll
                for (int i = 0; i < VG_MAX_KEYS; i++) k.w[i] = 0;
                uint32_t nm = 0;
                vgj_keys(X, j, k, nm);
                const int64_t g = gt_find_insert(L.gt, k, VGJ_NK, kt, nm, hash_k(k, VGJ_NK, nm));
                if (g < 0) {
                    if (m) spill_row(L, li, 0, -1);
                    else vgj_spill(L, li, failm[j]);
                    continue;
                }
#if VGJ_TRACK
                if (m) atomicMin((unsigned long long *)(L.gt.first_row + g), (unsigned long long)vgj_order(L, li, matched, j));
#endif
                vgj_global_update(L, g, X, j, m ? 0xFFFFFFFFu : failm[j]);
            }
        }
#endif
    }


#if VGJ_COMPACT
    flush_queue(qn);
#endif
    __syncthreads();
#if VGJ_PART_CTA && VGJ_PART_HOLES
    {
        // positions of this CTA's ranges that no row took (dropped rows)
        const uint32_t *pc = (const uint32_t *)(sm + VGJ_OFF_PCUR);
        for (int i = threadIdx.x; i < L.po.n_buckets; i += blockDim.x) {
            const uint64_t e = L.po.cta_off[(int64_t)i * gridDim.x + blockIdx.x + 1];
            for (uint64_t q = pc[i]; q < e; q++) {
                ulonglong2 *r = (ulonglong2 *)(L.po.rec + q * (uint64_t)L.po.rec_words);
                r[0] = make_ulonglong2(0ull, VG_PAGG_HOLE);
            }
        }
    }
#endif
    __shared__ Lay sl;
    if (threadIdx.x == 0) make_lay(L, (uint64_t)L.spill_cache_cap, sl);
    __syncthreads();
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
#if VGJ_DENSE && VGJ_LIVE_BY_CNT
        // every row counts in n(): a slot some row touched has a nonzero count
        if (((const uint32_t *)(sm + VGJ_LIVE_CNT))[i] == 0u) continue;
#else
        if (st[i] != 2u) continue;
#endif
        vgj_fix_bases(sm, i);
        if (!merge_entry(L, sm, cl, S, i)) spill_entry(L, sm, cl, S, i, sl);
    }
}
