// k_pagg.cu -- ahead-of-time kernels of the partitioned aggregation (many
// groups, one int64 key, key-ordered output; sm_103a):
//
//   sketch   one pass over the key column: a HyperLogLog estimate of the
//            distinct keys (4096 registers, Flajolet et al. 2007) and the
//            range of the keys' order words (key ^ 2^63);
//   hist     rows per key-range bucket (the bucket ranges of the records);
//   scan     bucket offsets and cursors;
//   refine   a bucket with more groups than one reducer CTA holds is split
//            by its own key range into 256 sub-buckets (records copied);
//   emit     the staged group results of a run of buckets, in bucket
//            order, compacted into output columns (validity bits OR-ed in at
//            the run's first output row).
//
// The first step proper (rows -> records) is the run-time specialised
// fused kernel in partition mode (jit_agg.cu), the second (records ->
// groups) the run-time specialised reducer (k_jit_pagg.cuh).  Together they
// replace the hash path of src/group_agg.c:155-281 for inputs whose group
// table would not fit on chip: every row is read once and written once as
// a record, every record read once, and all accumulation happens in shared
// memory instead of random atomics on a table in HBM.

#include <cmath>
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

constexpr int kHllBits = 12;
constexpr int kHllRegs = 1 << kHllBits;
constexpr int kHistSmemBuckets = 32768;     // bucket counters a CTA keeps in shared memory
constexpr int kThreads = 1024;

int grid_for(int64_t n, int per_cta) {
    int sms = vgk_num_sms();
    int64_t g = (n + per_cta - 1) / per_cta;
    int64_t cap = (int64_t)sms * 2;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

VG_DEV uint32_t bucket_of(uint64_t key, uint64_t omin, int shift, int nb) {
    const uint64_t ow = key ^ 0x8000000000000000ull;
    const uint64_t d = ow < omin ? 0ull : ((ow - omin) >> shift);
    return d >= (uint64_t)nb ? (uint32_t)(nb - 1) : (uint32_t)d;
}

// logical row i of a column view with an optional selection vector
VG_DEV int64_t phys_row(const int32_t *sel, int64_t i) { return sel ? (int64_t)__ldg(sel + i) : i; }

// Calls f(key) for the valid keys of logical rows [lo, hi) (sel: their
// physical rows), each thread taking four consecutive rows per step with
// two 16-byte loads when the column allows: enough loads in flight to keep
// a scan of the key column near HBM speed.  lo must be a multiple of 4.
template <typename F>
VG_DEV void for_valid_keys(const VgCol &key, int64_t lo, int64_t hi, const int32_t *sel, int64_t tid,
                           int64_t nthreads, F f) {
    const uint64_t *d = (const uint64_t *)key.data;
    const bool vec = !sel && (((uintptr_t)d & 15) == 0);
    for (int64_t r = lo + 4 * tid; r < hi; r += 4 * nthreads) {
        uint64_t k[4];
        int64_t row[4];
        if (vec && r + 4 <= hi) {
            const ulonglong2 a = __ldg((const ulonglong2 *)(d + r));
            const ulonglong2 b = __ldg((const ulonglong2 *)(d + r + 2));
            k[0] = a.x;
            k[1] = a.y;
            k[2] = b.x;
            k[3] = b.y;
#pragma unroll
            for (int j = 0; j < 4; j++) row[j] = r + j;
        } else {
#pragma unroll
            for (int j = 0; j < 4; j++) {
                row[j] = r + j < hi ? phys_row(sel, r + j) : -1;
                k[j] = row[j] >= 0 ? __ldg(d + row[j]) : 0;
            }
        }
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (row[j] >= 0 && vg_valid(key, row[j])) f(k[j]);
    }
}

// end of bucket b's records in region r (never past the bucket's range)
VG_DEV uint64_t rec_end(const VgPaggReduce &R, int r, int64_t b) {
    const uint64_t e = R.rend[r][b], e2 = R.roff[r][b + 1];
    return e < e2 ? e : e2;
}

VG_DEV void reduce_minmax(uint64_t lo, uint64_t hi, unsigned long long cnt, unsigned long long *mm) {
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t l2 = __shfl_xor_sync(0xFFFFFFFFu, lo, o);
        const uint64_t h2 = __shfl_xor_sync(0xFFFFFFFFu, hi, o);
        cnt += __shfl_xor_sync(0xFFFFFFFFu, cnt, o);
        lo = l2 < lo ? l2 : lo;
        hi = h2 > hi ? h2 : hi;
    }
    __shared__ unsigned long long wl[32], wh[32], wc[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { wl[warp] = lo; wh[warp] = hi; wc[warp] = cnt; }
    __syncthreads();
    if (warp == 0) {
        const int nw = (int)(blockDim.x >> 5);
        lo = lane < nw ? wl[lane] : ~0ull;
        hi = lane < nw ? wh[lane] : 0ull;
        cnt = lane < nw ? wc[lane] : 0ull;
        for (int o = 16; o > 0; o >>= 1) {
            const uint64_t l2 = __shfl_xor_sync(0xFFFFFFFFu, lo, o);
            const uint64_t h2 = __shfl_xor_sync(0xFFFFFFFFu, hi, o);
            cnt += __shfl_xor_sync(0xFFFFFFFFu, cnt, o);
            lo = l2 < lo ? l2 : lo;
            hi = h2 > hi ? h2 : hi;
        }
        if (lane == 0 && cnt) {
            atomicMin(mm, (unsigned long long)lo);
            atomicMax(mm + 1, (unsigned long long)hi);
            atomicAdd(mm + 2, cnt);
        }
    }
}

// mm: [0] min order word, [1] max order word, [2] valid keys (init ~0, 0, 0)
__global__ void __launch_bounds__(kThreads) sketch_kernel(VgCol key, int64_t n, const int32_t *sel, uint32_t *regs,
                                                          unsigned long long *mm) {
    __shared__ uint32_t r[kHllRegs];
    for (int i = threadIdx.x; i < kHllRegs; i += blockDim.x) r[i] = 0;
    __syncthreads();
    uint64_t lo = ~0ull, hi = 0;
    unsigned long long cnt = 0;
    for_valid_keys(key, 0, n, sel, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x,
                   [&](uint64_t k) {
                       const uint64_t ow = k ^ 0x8000000000000000ull;
                       lo = ow < lo ? ow : lo;
                       hi = ow > hi ? ow : hi;
                       cnt++;
                       const uint64_t h = vg_mix64(k);
                       const uint64_t w = h << kHllBits;
                       const uint32_t rank =
                           w ? (uint32_t)__clzll((long long)w) + 1u : (uint32_t)(64 - kHllBits + 1);
                       const uint32_t idx = (uint32_t)(h >> (64 - kHllBits));
                       if (rank > r[idx]) atomicMax(r + idx, rank);
                   });
    reduce_minmax(lo, hi, cnt, mm);
    __syncthreads();
    for (int i = threadIdx.x; i < kHllRegs; i += blockDim.x)
        if (r[i]) atomicMax(regs + i, r[i]);
}

__global__ void __launch_bounds__(kThreads) hist_kernel(VgCol key, int64_t n, const int32_t *sel, uint64_t omin,
                                                        int shift, int nb, uint32_t *cnt) {
    extern __shared__ uint32_t h[];
    const bool local = nb <= kHistSmemBuckets;
    if (local) {
        for (int i = threadIdx.x; i < nb; i += blockDim.x) h[i] = 0;
        __syncthreads();
    }
    for_valid_keys(key, 0, n, sel, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x,
                   [&](uint64_t k) {
                       const uint32_t b = bucket_of(k, omin, shift, nb);
                       if (local) atomicAdd(h + b, 1u);
                       else atomicAdd(cnt + b, 1u);
                   });
    if (local) {
        __syncthreads();
        for (int i = threadIdx.x; i < nb; i += blockDim.x)
            if (h[i]) atomicAdd(cnt + i, h[i]);
    }
}

// Valid keys per (bucket, CTA) over the fused kernel's tiles: CTA c counts
// tiles c, c + gridDim.x, ... of `tile` logical rows, as that kernel's CTA
// c processes them; m[b * gridDim.x + c].
__global__ void __launch_bounds__(kThreads) hist_cta_kernel(VgCol key, int64_t n, const int32_t *sel, uint64_t omin,
                                                            int shift, int nb, int64_t tile, uint32_t *m) {
    extern __shared__ uint32_t h[];
    for (int i = threadIdx.x; i < nb; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const int64_t ntiles = (n + tile - 1) / tile;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t r1 = (t + 1) * tile < n ? (t + 1) * tile : n;
        for_valid_keys(key, t * tile, r1, sel, threadIdx.x, blockDim.x,
                       [&](uint64_t k) { atomicAdd(h + bucket_of(k, omin, shift, nb), 1u); });
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x) m[(int64_t)i * gridDim.x + blockIdx.x] = h[i];
}

// Exclusive scan of n u32 counts into u64 offsets (out[n] = total), in
// three passes: chunk sums, their scan (one CTA), chunk scans.
constexpr int kScanChunk = kThreads * 16;

__global__ void __launch_bounds__(kThreads) scan_sums_kernel(const uint32_t *in, int64_t n, unsigned long long *sums) {
    const int64_t lo = (int64_t)blockIdx.x * kScanChunk;
    unsigned long long t = 0;
    for (int64_t i = lo + threadIdx.x; i < lo + kScanChunk && i < n; i += blockDim.x) t += in[i];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
    __shared__ unsigned long long w[32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += w[i];
        sums[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(kThreads) scan_chunks_kernel(const uint32_t *in, int64_t n,
                                                               const unsigned long long *sums, int64_t n_chunks,
                                                               uint64_t *out) {
    __shared__ unsigned long long base, w[32];
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int64_t c = 0; c < blockIdx.x; c++) s += sums[c];   // few chunks: sums are L2-resident
        base = s;
        if (blockIdx.x == n_chunks - 1) out[n] = s + sums[blockIdx.x];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t lo = (int64_t)blockIdx.x * kScanChunk;
    for (int64_t b0 = lo; b0 < lo + kScanChunk && b0 < n; b0 += blockDim.x) {
        const int64_t i = b0 + threadIdx.x;
        const unsigned long long v = i < n ? in[i] : 0ull;
        unsigned long long x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) w[warp] = x;
        __syncthreads();
        if (warp == 0) {
            const int nw = (int)(blockDim.x >> 5);
            unsigned long long y = lane < nw ? w[lane] : 0ull;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long z = __shfl_up_sync(0xFFFFFFFFu, y, o);
                if (lane >= o) y += z;
            }
            if (lane < nw) w[lane] = y;
        }
        __syncthreads();
        const unsigned long long excl = base + (warp ? w[warp - 1] : 0ull) + x - v;
        if (i < n) out[i] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) base = excl + v;
        __syncthreads();
    }
}

// One CTA: off[b] = sum of cnt[0..b), off[nb] = total; cursor[b * cstride]
// = off[b] (cursor optional).  cnt == nullptr: counts are rend[b] - roff[b] summed
// over the regions of R (bucket sizes of a set of regions).
__global__ void __launch_bounds__(kThreads) scan_kernel(const uint32_t *cnt, VgPaggReduce R, int64_t nb,
                                                        uint64_t *off, unsigned long long *cursor, int cstride) {
    __shared__ unsigned long long part[kThreads];
    const int64_t per = (nb + blockDim.x - 1) / blockDim.x;
    const int64_t lo = (int64_t)threadIdx.x * per;
    const int64_t hi = lo + per < nb ? lo + per : nb;
    auto count = [&](int64_t b) -> unsigned long long {
        if (cnt) return cnt[b];
        unsigned long long t = 0;
        for (int r = 0; r < R.n_regions; r++) t += rec_end(R, r, b) - R.roff[r][b];
        return t;
    };
    unsigned long long s = 0;
    for (int64_t b = lo; b < hi; b++) s += count(b);
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long run = 0;
        for (int i = 0; i < (int)blockDim.x; i++) {
            const unsigned long long x = part[i];
            part[i] = run;
            run += x;
        }
        off[nb] = run;
    }
    __syncthreads();
    unsigned long long run = part[threadIdx.x];
    for (int64_t b = lo; b < hi; b++) {
        off[b] = run;
        if (cursor) cursor[b * cstride] = run;
        run += count(b);
    }
}

__global__ void cursor_compact_kernel(const unsigned long long *padded, int stride, int64_t nb,
                                      unsigned long long *dense) {
    const int64_t st = (int64_t)gridDim.x * blockDim.x;
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += st) dense[b] = padded[b * stride];
}

// ---------------------------------------------------------------------
// refinement of one bucket (records spread over the regions of R)
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) rec_minmax_kernel(VgPaggReduce R, int b, unsigned long long *mm) {
    uint64_t lo = ~0ull, hi = 0;
    unsigned long long cnt = 0;
    for (int r = 0; r < R.n_regions; r++) {
        const uint64_t a = R.roff[r][b], e = rec_end(R, r, b);
        const int64_t stride = (int64_t)gridDim.x * blockDim.x;
        for (uint64_t p = a + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < e; p += stride) {
            if (__ldg(R.rec[r] + p * R.rec_words + 1) & VG_PAGG_HOLE) continue;
            const uint64_t ow = __ldg(R.rec[r] + p * R.rec_words) ^ 0x8000000000000000ull;
            lo = ow < lo ? ow : lo;
            hi = ow > hi ? ow : hi;
            cnt++;
        }
    }
    reduce_minmax(lo, hi, cnt, mm);
}

__global__ void __launch_bounds__(kThreads) rec_hist_kernel(VgPaggReduce R, int b, uint64_t omin, int shift, int nb,
                                                            uint32_t *cnt) {
    __shared__ uint32_t h[256];
    for (int i = threadIdx.x; i < nb; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (int r = 0; r < R.n_regions; r++) {
        const uint64_t a = R.roff[r][b], e = rec_end(R, r, b);
        const int64_t stride = (int64_t)gridDim.x * blockDim.x;
        for (uint64_t p = a + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < e; p += stride)
            if (!(__ldg(R.rec[r] + p * R.rec_words + 1) & VG_PAGG_HOLE))
                atomicAdd(h + bucket_of(__ldg(R.rec[r] + p * R.rec_words), omin, shift, nb), 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
        if (h[i]) atomicAdd(cnt + i, h[i]);
}

__global__ void __launch_bounds__(kThreads) rec_scatter_kernel(VgPaggReduce R, int b, uint64_t omin, int shift,
                                                               int nb, unsigned long long *cursor, const uint64_t *end,
                                                               uint64_t *out, uint32_t *err) {
    const int rw = R.rec_words;
    for (int r = 0; r < R.n_regions; r++) {
        const uint64_t a = R.roff[r][b], e = rec_end(R, r, b);
        const int64_t stride = (int64_t)gridDim.x * blockDim.x;
        for (uint64_t p = a + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < e; p += stride) {
            const uint64_t *src = R.rec[r] + p * rw;
            if (__ldg(src + 1) & VG_PAGG_HOLE) continue;
            const uint32_t sb = bucket_of(__ldg(src), omin, shift, nb);
            const unsigned long long pos = atomicAdd(cursor + sb, 1ull);
            if (pos >= end[sb]) { atomicOr(err, VG_ERR_FULL); continue; }
            for (int w = 0; w < rw; w++) out[pos * rw + w] = __ldg(src + w);
        }
    }
}

// ---------------------------------------------------------------------
// emit: staged groups -> output columns
// ---------------------------------------------------------------------
struct EmitArgs {
    int64_t n_leaves;
    const uint64_t *leaf_stage;   // staging position of each leaf's first group
    const uint64_t *leaf_out;     // output position of each leaf's first group (n_leaves + 1 entries)
    int64_t n_groups;             // output rows (the NA group included)
    int32_t has_na;
    int32_t n_out;
    uint64_t na_stage;
    uint64_t out_base;            // validity bit of output row j: out_base + j (OR-ed into zeroed words)
    const uint64_t *st_key;
    const uint32_t *st_ok;
    const double *st_out[VG_MAX_OUTS];
    uint64_t *key_out;
    uint32_t *key_valid;
    double *out[VG_MAX_OUTS];
    uint32_t *out_valid[VG_MAX_OUTS];
};

__global__ void __launch_bounds__(256) emit_kernel(const __grid_constant__ EmitArgs A) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n_pad = (A.n_groups + 31) & ~31ll;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n_pad; j += stride) {
        const bool in = j < A.n_groups;
        const bool na = in && A.has_na && j == A.n_groups - 1;
        uint64_t src = 0;
        if (in && !na) {
            int64_t lo = 0, hi = A.n_leaves - 1;   // last leaf whose first output position <= j
            while (lo < hi) {
                const int64_t mid = (lo + hi + 1) >> 1;
                if (__ldg(A.leaf_out + mid) <= (uint64_t)j) lo = mid;
                else hi = mid - 1;
            }
            src = __ldg(A.leaf_stage + lo) + ((uint64_t)j - __ldg(A.leaf_out + lo));
        } else if (na) {
            src = A.na_stage;
        }
        if (in) A.key_out[j] = na ? 0ull : A.st_key[src];
        // a warp's 32 validity bits land at bit out_base + j0 (j0 = j - lane)
        const uint64_t bit0 = A.out_base + (uint64_t)(j - lane);
        auto put = [&](uint32_t *v, uint32_t m) {
            if (lane != 0 || !m) return;
            const uint64_t w = ((uint64_t)m) << (bit0 & 31);
            atomicOr(v + (bit0 >> 5), (uint32_t)w);
            if (w >> 32) atomicOr(v + (bit0 >> 5) + 1, (uint32_t)(w >> 32));
        };
        put(A.key_valid, __ballot_sync(0xFFFFFFFFu, in && !na));
        const uint32_t okb = in ? A.st_ok[src] : 0u;
        for (int o = 0; o < A.n_out; o++) {
            const bool ok = (okb >> o) & 1u;
            if (in) A.out[o][j] = ok ? A.st_out[o][src] : 0.0;
            put(A.out_valid[o], __ballot_sync(0xFFFFFFFFu, in && ok));
        }
    }
}

// Check of vg_window6_to_double against vg_digits_to_double on seeded
// random windows (several magnitude classes, both signs, every base).
__global__ void window_selftest_kernel(int64_t n, uint64_t seed, unsigned long long *bad) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t x = vg_mix64(seed ^ (uint64_t)i) | 1;
        auto next = [&]() {
            x ^= x << 13;
            x ^= x >> 7;
            x ^= x << 17;
            return x;
        };
        const int base = (int)(next() % 61);
        const int cls = (int)(next() % 6);
        int64_t w[6];
        for (int k = 0; k < 6; k++) {
            const uint64_t r = next();
            int64_t v;
            if (cls == 0) v = (int64_t)(r >> 2) - (int64_t)(1ull << 61);               // full-size, mixed signs
            else if (cls == 1) v = (int64_t)(r & 0xFFFFF) - 0x80000;                   // small
            else if (cls == 2) v = k == (int)(r % 6) ? (int64_t)(r >> 3) : 0;          // one digit
            else if (cls == 3) v = (int64_t)(r >> 33);                                 // 31-bit positive
            else if (cls == 4) v = -(int64_t)(r >> 33);                                // 31-bit negative
            else v = (k < 2) ? (int64_t)(r & 0xFFFF) : 0;                              // tiny (exact range)
            w[k] = v;
        }
        int64_t full[VG_LACC_WORDS];
        for (int k = 0; k < VG_LACC_WORDS; k++) full[k] = 0;
        for (int k = 0; k < 6; k++) full[base + k] = w[k];
        const double a = vg_window6_to_double(w, base);
        const double b = vg_digits_to_double(full, VG_LACC_WORDS, 0);
        if (__double_as_longlong(a) != __double_as_longlong(b)) atomicAdd(bad, 1ull);
    }
}

}  // namespace

extern "C" {

const char *vgk_pagg_last_error(void) { return g_err; }

// Mismatches of the register-only window rounding against the general
// digit rounding on n seeded windows (-1 on a CUDA error).
long long vgpu_pagg_window_selftest(long long n, unsigned long long seed) {
    unsigned long long *d = nullptr, h = 0;
    if (cudaMalloc(&d, 8) != cudaSuccess) return -1;
    cudaMemset(d, 0, 8);
    window_selftest_kernel<<<grid_for(n, 256), 256>>>(n, seed, d);
    vg_launch_counter++;
    cudaMemcpy(&h, d, 8, cudaMemcpyDeviceToHost);
    const cudaError_t e = cudaGetLastError();
    cudaFree(d);
    return e == cudaSuccess ? (long long)h : -1;
}

int vgk_pagg_sketch(const VgCol *key, int64_t n, const int32_t *sel, uint32_t *d_regs, unsigned long long *d_mm,
                    double *h_distinct, uint64_t *h_mm, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    const unsigned long long init[3] = {~0ull, 0ull, 0ull};
    cudaMemsetAsync(d_regs, 0, kHllRegs * 4, st);
    cudaMemcpyAsync(d_mm, init, sizeof(init), cudaMemcpyHostToDevice, st);
    if (n > 0) {
        sketch_kernel<<<grid_for(n, kThreads * 8), kThreads, 0, st>>>(*key, n, sel, d_regs, d_mm);
        vg_launch_counter++;
    }
    uint32_t regs[kHllRegs];
    cudaMemcpyAsync(regs, d_regs, sizeof(regs), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(h_mm, d_mm, 3 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st);
    if (check(cudaStreamSynchronize(st), "pagg sketch")) return -1;
    // HyperLogLog estimate with the small-range (linear counting) correction
    const double m = (double)kHllRegs;
    double z = 0.0;
    int zeros = 0;
    for (int i = 0; i < kHllRegs; i++) {
        z += ldexp(1.0, -(int)regs[i]);
        if (regs[i] == 0) zeros++;
    }
    double e = (0.7213 / (1.0 + 1.079 / m)) * m * m / z;
    if (e <= 2.5 * m && zeros > 0) e = m * log(m / (double)zeros);
    *h_distinct = e;
    return 0;
}

int vgk_pagg_hist(const VgCol *key, int64_t n, const int32_t *sel, uint64_t omin, int shift, int nb, uint32_t *d_cnt,
                  vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    cudaMemsetAsync(d_cnt, 0, (size_t)nb * 4, st);
    if (n > 0) {
        const size_t smem = nb <= kHistSmemBuckets ? (size_t)nb * 4 : 0;
        static int attr_set = 0;
        if (!attr_set) {
            cudaFuncSetAttribute(hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kHistSmemBuckets * 4);
            attr_set = 1;
        }
        hist_kernel<<<grid_for(n, kThreads * 8), kThreads, smem, st>>>(*key, n, sel, omin, shift, nb, d_cnt);
        vg_launch_counter++;
    }
    return check(cudaGetLastError(), "pagg hist");
}

int vgk_pagg_scan(const uint32_t *d_cnt, const VgPaggReduce *regions, int64_t nb, uint64_t *d_off,
                  unsigned long long *d_cursor, int cursor_stride, vg_stream_t s) {
    VgPaggReduce R;
    memset(&R, 0, sizeof(R));
    if (regions) R = *regions;
    scan_kernel<<<1, kThreads, 0, (cudaStream_t)s>>>(d_cnt, R, nb, d_off, d_cursor, cursor_stride);
    vg_launch_counter++;
    return check(cudaGetLastError(), "pagg scan");
}

int vgk_pagg_hist_cta(const VgCol *key, int64_t n, const int32_t *sel, uint64_t omin, int shift, int nb, int grid,
                      int64_t tile, uint32_t *d_m, vg_stream_t s) {
    if (nb > kHistSmemBuckets) {
        snprintf(g_err, sizeof(g_err), "pagg hist: at most %d buckets per CTA", kHistSmemBuckets);
        return -1;
    }
    static int attr_set = 0;
    if (!attr_set) {
        cudaFuncSetAttribute(hist_cta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kHistSmemBuckets * 4);
        attr_set = 1;
    }
    hist_cta_kernel<<<grid, kThreads, (size_t)nb * 4, (cudaStream_t)s>>>(*key, n, sel, omin, shift, nb, tile, d_m);
    vg_launch_counter++;
    return check(cudaGetLastError(), "pagg hist per CTA");
}

// out[0..n]: exclusive scan of in[0..n) (out[n] = total); d_sums: scratch
// of one word per 16Ki entries
int vgk_scan_u32_u64(const uint32_t *in, int64_t n, uint64_t *out, unsigned long long *d_sums, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    const int64_t chunks = (n + kScanChunk - 1) / kScanChunk;
    if (chunks == 0) {
        cudaMemsetAsync(out, 0, 8, st);
        return check(cudaGetLastError(), "scan");
    }
    scan_sums_kernel<<<(int)chunks, kThreads, 0, st>>>(in, n, d_sums);
    scan_chunks_kernel<<<(int)chunks, kThreads, 0, st>>>(in, n, d_sums, chunks, out);
    vg_launch_counter += 2;
    return check(cudaGetLastError(), "scan");
}

// dense[b] = padded[b * stride]: the record ends after the partition pass
int vgk_pagg_cursor_compact(const unsigned long long *padded, int stride, int64_t nb, unsigned long long *dense,
                            vg_stream_t s) {
    cursor_compact_kernel<<<grid_for(nb, 256), 256, 0, (cudaStream_t)s>>>(padded, stride, nb, dense);
    vg_launch_counter++;
    return check(cudaGetLastError(), "pagg cursors");
}

int vgk_pagg_rec_minmax(const VgPaggReduce *R, int b, uint64_t rows, unsigned long long *d_mm, uint64_t *h_mm,
                        vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    const unsigned long long init[3] = {~0ull, 0ull, 0ull};
    cudaMemcpyAsync(d_mm, init, sizeof(init), cudaMemcpyHostToDevice, st);
    rec_minmax_kernel<<<grid_for((int64_t)rows, kThreads * 4), kThreads, 0, st>>>(*R, b, d_mm);
    vg_launch_counter++;
    cudaMemcpyAsync(h_mm, d_mm, 3 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st);
    return check(cudaStreamSynchronize(st), "pagg refine range");
}

int vgk_pagg_rec_split(const VgPaggReduce *R, int b, uint64_t rows, uint64_t omin, int shift, int nb, uint32_t *d_cnt,
                       uint64_t *d_off, unsigned long long *d_cursor, uint64_t *d_out, uint32_t *d_err,
                       vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    if (nb > 256) {
        snprintf(g_err, sizeof(g_err), "pagg refine: at most 256 sub-buckets");
        return -1;
    }
    cudaMemsetAsync(d_cnt, 0, (size_t)nb * 4, st);
    const int grid = grid_for((int64_t)rows, kThreads * 4);
    rec_hist_kernel<<<grid, kThreads, 0, st>>>(*R, b, omin, shift, nb, d_cnt);
    vg_launch_counter++;
    if (vgk_pagg_scan(d_cnt, nullptr, nb, d_off, d_cursor, 1, s)) return -1;
    rec_scatter_kernel<<<grid, kThreads, 0, st>>>(*R, b, omin, shift, nb, d_cursor, d_off + 1, d_out, d_err);
    vg_launch_counter++;
    return check(cudaGetLastError(), "pagg refine split");
}

int vgk_pagg_emit(int64_t n_leaves, const uint64_t *d_leaf_stage, const uint64_t *d_leaf_out, int64_t n_groups,
                  int has_na, uint64_t na_stage, const uint64_t *st_key, const uint32_t *st_ok,
                  const double *const *st_out, int n_out, uint64_t *key_out, uint32_t *key_valid, double **out,
                  uint32_t **out_valid, uint64_t out_base, vg_stream_t s) {
    if (n_groups <= 0) return 0;
    if (n_out > VG_MAX_OUTS) {
        snprintf(g_err, sizeof(g_err), "pagg emit: too many outputs");
        return -1;
    }
    EmitArgs A;
    memset(&A, 0, sizeof(A));
    A.n_leaves = n_leaves;
    A.leaf_stage = d_leaf_stage;
    A.leaf_out = d_leaf_out;
    A.n_groups = n_groups;
    A.has_na = has_na;
    A.n_out = n_out;
    A.na_stage = na_stage;
    A.out_base = out_base;
    A.st_key = st_key;
    A.st_ok = st_ok;
    A.key_out = key_out;
    A.key_valid = key_valid;
    for (int o = 0; o < n_out; o++) {
        A.st_out[o] = st_out[o];
        A.out[o] = out[o];
        A.out_valid[o] = out_valid[o];
    }
    const int sms = vgk_num_sms();
    int64_t grid = (n_groups + 255) / 256;
    if (grid > (int64_t)sms * 8) grid = (int64_t)sms * 8;
    vg_prof_begin(VG_PROF_FINISH, (cudaStream_t)s);
    emit_kernel<<<(int)grid, 256, 0, (cudaStream_t)s>>>(A);
    vg_launch_counter++;
    vg_prof_end(VG_PROF_FINISH, (cudaStream_t)s);
    return check(cudaGetLastError(), "pagg emit");
}

}  // extern "C"
