// k_sort.cu -- device-wide building blocks: a stable LSD radix sort of
// (64-bit key, 32-bit value) pairs and exclusive prefix sums (sm_103a).
// The group order built on them is the reference's sorted path's:
// ascending key, NA last (compare_value, src/sort.c:32-38;
// sorted_agg_next_batch, src/group_agg.c:466-585).

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

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 16;
constexpr int kRadixTile = kRadixThreads * kRadixItems;

__global__ void radix_hist_kernel(const uint64_t *keys, int64_t n, int shift, uint32_t *hist,
                                  int n_tiles) {
    __shared__ uint32_t h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    int64_t t0 = (int64_t)blockIdx.x * kRadixTile;
    for (int i = threadIdx.x; i < kRadixTile; i += blockDim.x) {
        int64_t idx = t0 + i;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 0xFF], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(int64_t)d * n_tiles + blockIdx.x] = h[d];
}

// exclusive scan, in place, of `total` uint32 counts (one CTA; the counts
// are small: 256 per tile of 4096 items)
__global__ void __launch_bounds__(1024) scan_u32_one_cta(uint32_t *v, int64_t total) {
    __shared__ uint32_t part[1024];
    int64_t per = (total + blockDim.x - 1) / blockDim.x;
    int64_t lo = (int64_t)threadIdx.x * per, hi = lo + per;
    if (hi > total) hi = total;
    if (lo > total) lo = total;
    uint32_t s = 0;
    for (int64_t i = lo; i < hi; i++) s += v[i];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int i = 0; i < (int)blockDim.x; i++) { uint32_t x = part[i]; part[i] = run; run += x; }
    }
    __syncthreads();
    uint32_t run = part[threadIdx.x];
    for (int64_t i = lo; i < hi; i++) { uint32_t x = v[i]; v[i] = run; run += x; }
}

__global__ void __launch_bounds__(kRadixThreads)
radix_scatter_kernel(const uint64_t *keys_in, const int32_t *vals_in, int64_t n, int shift,
                     const uint32_t *offsets, int n_tiles, uint64_t *keys_out, int32_t *vals_out) {
    __shared__ uint32_t cnt[256];
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[kRadixThreads / 32][256];
    int64_t t0 = (int64_t)blockIdx.x * kRadixTile;
    for (int d = threadIdx.x; d < 256; d += blockDim.x) {
        cnt[d] = 0;
        base[d] = offsets[(int64_t)d * n_tiles + blockIdx.x];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int r = 0; r < kRadixItems; r++) {
        int64_t idx = t0 + (int64_t)r * kRadixThreads + threadIdx.x;
        bool in = idx < n;
        uint64_t key = in ? keys_in[idx] : 0;
        uint32_t d = in ? (uint32_t)((key >> shift) & 0xFF) : 256u + (uint32_t)lane;
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        uint32_t lower = __popc(peers & ((1u << lane) - 1));
        for (int i = threadIdx.x; i < (kRadixThreads / 32) * 256; i += blockDim.x)
            (&wcnt[0][0])[i] = 0;
        __syncthreads();
        if (in && lower == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (in) {
            uint32_t before = 0;
            for (int w = 0; w < warp; w++) before += wcnt[w][d];
            uint64_t pos = (uint64_t)base[d] + cnt[d] + before + lower;
            keys_out[pos] = key;
            vals_out[pos] = vals_in[idx];
        }
        __syncthreads();
        for (int dd = threadIdx.x; dd < 256; dd += blockDim.x) {
            uint32_t s = 0;
            for (int w = 0; w < kRadixThreads / 32; w++) s += wcnt[w][dd];
            cnt[dd] += s;
        }
        __syncthreads();
    }
}

// ---- exclusive scan of int32 counts into int64 offsets ----
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads)
tile_sums_kernel(const int32_t *in, int64_t n, int64_t *sums) {
    __shared__ int64_t part[kScanThreads / 32];
    int64_t t0 = (int64_t)blockIdx.x * kScanTile;
    int64_t s = 0;
    for (int i = threadIdx.x; i < kScanTile; i += blockDim.x) {
        int64_t idx = t0 + i;
        if (idx < n) s += in[idx];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int w = 0; w < kScanThreads / 32; w++) t += part[w];
        sums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(1024) scan_i64_one_cta(int64_t *v, int64_t total, int64_t *grand) {
    __shared__ int64_t part[1024];
    int64_t per = (total + blockDim.x - 1) / blockDim.x;
    int64_t lo = (int64_t)threadIdx.x * per, hi = lo + per;
    if (hi > total) hi = total;
    if (lo > total) lo = total;
    int64_t s = 0;
    for (int64_t i = lo; i < hi; i++) s += v[i];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t run = 0;
        for (int i = 0; i < (int)blockDim.x; i++) { int64_t x = part[i]; part[i] = run; run += x; }
        if (grand) *grand = run;
    }
    __syncthreads();
    int64_t run = part[threadIdx.x];
    for (int64_t i = lo; i < hi; i++) { int64_t x = v[i]; v[i] = run; run += x; }
}

__global__ void __launch_bounds__(kScanThreads)
tile_scan_kernel(const int32_t *in, int64_t n, const int64_t *tile_base, int64_t *out) {
    __shared__ int64_t wsum[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t t0 = (int64_t)blockIdx.x * kScanTile;
    // each thread owns kScanItems consecutive items
    int64_t i0 = t0 + (int64_t)threadIdx.x * kScanItems;
    int32_t v[kScanItems];
    int64_t local = 0;
    for (int k = 0; k < kScanItems; k++) {
        v[k] = (i0 + k < n) ? in[i0 + k] : 0;
        local += v[k];
    }
    int64_t x = local;
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    int64_t wb = 0;
    for (int w = 0; w < warp; w++) wb += wsum[w];
    int64_t run = tile_base[blockIdx.x] + wb + (x - local);
    for (int k = 0; k < kScanItems; k++) {
        if (i0 + k < n) out[i0 + k] = run;
        run += v[k];
    }
}

// ---- arrange(): the permutation of a stable multi-key sort ----

// The order word of a valid value (its order is the reference's value
// comparison, src/sort.c:32-71): int64 with the sign bit flipped; a double
// as its order-preserving bit image with -0 taken as +0 (equal, so ties
// keep their input order); a bool's byte.  Descending: the word inverted.
__device__ __forceinline__ uint64_t sort_word(const VgCol &c, int64_t r, int desc) {
    uint64_t w;
    if (c.type == VEC_BOOL) {
        w = (uint64_t)__ldg((const uint8_t *)c.data + r);
    } else {
        uint64_t b = vg_load_bits(c, r);
        if (c.type == VEC_DOUBLE) {
            if (b == 0x8000000000000000ull) b = 0;
            w = (b >> 63) ? ~b : (b | 0x8000000000000000ull);
        } else {
            w = b ^ 0x8000000000000000ull;
        }
    }
    return desc ? ~w : w;
}

// words[i] = the order word of row perm[i] (0 for NA); stats[0] |= the bits
// in which valid words differ from the first row's, stats[1] += NA rows
__global__ void sort_words_kernel(VgCol c, const int32_t *perm, int64_t n, int desc, uint64_t *words,
                                  unsigned long long *stats) {
    const int64_t r0 = __ldg(perm);
    const uint64_t wref = vg_valid(c, r0) ? sort_word(c, r0, desc) : 0ull;
    unsigned long long diff = 0, na = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int64_t r = __ldg(perm + i);
        uint64_t w = 0;
        if (vg_valid(c, r)) {
            w = sort_word(c, r, desc);
            diff |= w ^ wref;
        } else {
            na++;
        }
        words[i] = w;
    }
    for (int o = 16; o > 0; o >>= 1) {
        diff |= __shfl_xor_sync(0xFFFFFFFFu, diff, o);
        na += __shfl_xor_sync(0xFFFFFFFFu, na, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (diff) atomicOr(stats, diff);
        if (na) atomicAdd(stats + 1, na);
    }
}

// NA placement of row perm[i]: ascending puts NA after every value (flag
// 1), descending before them (flag 0 for NA), src/sort.c:38-40
__global__ void sort_naflag_kernel(VgCol c, const int32_t *perm, int64_t n, int desc, uint64_t *flags) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const bool v = vg_valid(c, __ldg(perm + i));
        flags[i] = desc ? (v ? 1ull : 0ull) : (v ? 0ull : 1ull);
    }
}

__global__ void iota_kernel(int32_t *perm, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) perm[i] = (int32_t)i;
}

}  // namespace

extern "C" {

const char *vgk_sort_last_error(void) { return g_err; }

size_t vgk_sort_rows_scratch(int64_t n) {
    const int64_t m = n > 0 ? n : 1;
    return a256((size_t)m * 8) + vgk_sort_pairs_scratch(m) + 256;
}

// perm (n int32 entries) := the stable order of rows 0..n-1 by the keys
// (cols[key_col[k]], descending desc[k]), the first key most significant:
// least significant key first, each key a radix sort of its order words
// over the bits in which they differ, then, if the key has NA rows, a
// one-bit pass that moves them after (ascending) or before (descending)
// the values.  Every pass is stable, as the reference's merge sort is
// (src/sort.c:97-116).
int vgk_sort_rows(const VgCol *cols, const int *key_col, const int *desc, int n_keys, int32_t *perm, int64_t n,
                  void *scratch, size_t scratch_bytes, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    if (n <= 0) return 0;
    if (scratch_bytes < vgk_sort_rows_scratch(n)) {
        snprintf(g_err, sizeof(g_err), "sort scratch too small");
        return -1;
    }
    char *p = (char *)scratch;
    uint64_t *words = (uint64_t *)p; p += a256((size_t)n * 8);
    void *pair_scratch = p; p += vgk_sort_pairs_scratch(n);
    unsigned long long *stats = (unsigned long long *)p;
    const int grid = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    iota_kernel<<<grid, 256, 0, st>>>(perm, n);
    vg_launch_counter++;
    for (int k = n_keys - 1; k >= 0; k--) {
        const VgCol &c = cols[key_col[k]];
        if (check(cudaMemsetAsync(stats, 0, 16, st), "sort")) return -1;
        sort_words_kernel<<<grid, 256, 0, st>>>(c, perm, n, desc[k], words, stats);
        vg_launch_counter++;
        unsigned long long h[2];
        if (check(cudaMemcpyAsync(h, stats, 16, cudaMemcpyDeviceToHost, st), "sort")) return -1;
        if (check(cudaStreamSynchronize(st), "sort")) return -1;
        int bits = 0;
        while (bits < 64 && (h[0] >> bits)) bits++;
        if (bits > 0 && vgk_sort_pairs(words, perm, n, bits, pair_scratch, vgk_sort_pairs_scratch(n), s) != 0)
            return -1;
        if (h[1] > 0) {
            sort_naflag_kernel<<<grid, 256, 0, st>>>(c, perm, n, desc[k], words);
            vg_launch_counter++;
            if (vgk_sort_pairs(words, perm, n, 1, pair_scratch, vgk_sort_pairs_scratch(n), s) != 0) return -1;
        }
    }
    return check(cudaGetLastError(), "sort");
}

size_t vgk_sort_pairs_scratch(int64_t n) {
    int64_t tiles = (n + kRadixTile - 1) / kRadixTile;
    if (tiles < 1) tiles = 1;
    return a256((size_t)n * 8) + a256((size_t)n * 4) + a256((size_t)tiles * 256 * 4);
}

// Stable ascending sort of keys (only the low key_bits bits are looked at)
// carrying vals; the result is left in keys / vals.
int vgk_sort_pairs(uint64_t *keys, int32_t *vals, int64_t n, int key_bits, void *scratch,
                   size_t scratch_bytes, vg_stream_t s) {
    if (n <= 1) return 0;
    if (scratch_bytes < vgk_sort_pairs_scratch(n)) {
        snprintf(g_err, sizeof(g_err), "sort scratch too small");
        return -1;
    }
    cudaStream_t st = (cudaStream_t)s;
    int64_t tiles = (n + kRadixTile - 1) / kRadixTile;
    char *p = (char *)scratch;
    uint64_t *k1 = (uint64_t *)p; p += a256((size_t)n * 8);
    int32_t *v1 = (int32_t *)p; p += a256((size_t)n * 4);
    uint32_t *hist = (uint32_t *)p;
    uint64_t *kin = keys, *kout = k1;
    int32_t *vin = vals, *vout = v1;
    int passes = (key_bits + 7) / 8;
    for (int d = 0; d < passes; d++) {
        { radix_hist_kernel<<<(int)tiles, kRadixThreads, 0, st>>>(kin, n, d * 8, hist, (int)tiles); vg_launch_counter++; }
        { scan_u32_one_cta<<<1, 1024, 0, st>>>(hist, tiles * 256); vg_launch_counter++; }
        { radix_scatter_kernel<<<(int)tiles, kRadixThreads, 0, st>>>(kin, vin, n, d * 8, hist, (int)tiles,
                                                                   kout, vout); vg_launch_counter++; }
        uint64_t *tk = kin; kin = kout; kout = tk;
        int32_t *tv = vin; vin = vout; vout = tv;
    }
    if (kin != keys) {
        cudaMemcpyAsync(keys, kin, (size_t)n * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(vals, vin, (size_t)n * 4, cudaMemcpyDeviceToDevice, st);
    }
    return check(cudaGetLastError(), "radix sort");
}

size_t vgk_scan_scratch(int64_t n) {
    int64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles < 1) tiles = 1;
    return a256((size_t)tiles * 8) + 256;
}

// out[i] = sum(in[0..i)), *d_total = sum(in) (device pointer, may be NULL)
int vgk_exclusive_scan(const int32_t *in, int64_t n, int64_t *out, int64_t *d_total, void *scratch,
                       size_t scratch_bytes, vg_stream_t s) {
    if (n <= 0) {
        if (d_total) cudaMemsetAsync(d_total, 0, 8, (cudaStream_t)s);
        return 0;
    }
    if (scratch_bytes < vgk_scan_scratch(n)) {
        snprintf(g_err, sizeof(g_err), "scan scratch too small");
        return -1;
    }
    cudaStream_t st = (cudaStream_t)s;
    int64_t tiles = (n + kScanTile - 1) / kScanTile;
    int64_t *sums = (int64_t *)scratch;
    { tile_sums_kernel<<<(int)tiles, kScanThreads, 0, st>>>(in, n, sums); vg_launch_counter++; }
    { scan_i64_one_cta<<<1, 1024, 0, st>>>(sums, tiles, d_total); vg_launch_counter++; }
    { tile_scan_kernel<<<(int)tiles, kScanThreads, 0, st>>>(in, n, sums, out); vg_launch_counter++; }
    return check(cudaGetLastError(), "scan");
}

}  // extern "C"
