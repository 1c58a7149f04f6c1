// k_strings.cu -- string columns on the device (sm_103a).
//
// A VEC_STRING column on the device is one 16-byte VgStrView per row
// (length, big-endian 4-byte prefix, pointer to the bytes); the bytes stay
// where the batch's upload put them.  This file builds views from the
// reference's offsets + bytes layout (src/types.h:56-60), packs views back
// into offsets + bytes for the host, and keeps string dictionaries: a
// device hash table mapping each distinct string to a dense int64 code, so
// that string group keys and join keys run through the integer key paths
// (the reference hashes and compares the bytes themselves,
// src/hash.c:35-43, 58-66).

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

constexpr uint32_t kEmpty = 0xFFFFFFFFu;
constexpr uint32_t kBusy = 0xFFFFFFFEu;

VG_DEV VgStrView load_view(const VgCol &c, int64_t p) {
    const ulonglong2 w = __ldg((const ulonglong2 *)c.data + p);
    VgStrView v;
    v.len = (uint32_t)w.x;
    v.pre = (uint32_t)(w.x >> 32);
    v.ptr = (const char *)w.y;
    return v;
}

// 64-bit hash of a byte string: 8-byte little-endian words through a
// multiply-xorshift mixer, the length folded in first
VG_DEV uint64_t str_hash(const char *p, uint32_t len) {
    uint64_t h = 0x9E3779B97F4A7C15ull ^ (uint64_t)len;
    uint32_t i = 0;
    for (; i + 8 <= len; i += 8) {
        uint64_t w = 0;
        for (int k = 0; k < 8; k++) w |= (uint64_t)(unsigned char)p[i + k] << (8 * k);
        h = (h ^ w) * 0xFF51AFD7ED558CCDull;
        h ^= h >> 32;
    }
    // the tail: up to 7 bytes, each read at a clamped position inside the
    // string and masked
    uint64_t w = 0;
    if (i < len) {
        const uint32_t last = len - 1;
        for (uint32_t k = 0; k < 8; k++) {
            const uint32_t at = i + k;
            const uint64_t b = (uint64_t)(unsigned char)p[at < last ? at : last];
            w |= (at < len ? b : 0ull) << (8 * k);
        }
    }
    h = (h ^ w) * 0xC4CEB9FE1A85EC53ull;
    h ^= h >> 29;
    h *= 0xFF51AFD7ED558CCDull;
    h ^= h >> 32;
    return h;
}

// views over the reference's layout: row i is bytes [offs[i], offs[i+1]),
// bytes[0] being the byte at offset `base`
__global__ void views_kernel(const int64_t *offs, int64_t base, const char *bytes, int64_t n, VgStrView *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int64_t a = offs[i], b = offs[i + 1];
        out[i] = vg_str_view(bytes + (a - base), (uint32_t)(b - a));
    }
}

// lengths of rows idx[j] (or j) and the validity words of the packed column
__global__ void lengths_kernel(VgCol c, const int32_t *idx, int64_t n, int32_t *len, uint32_t *out_valid) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n_pad = (n + 31) & ~31ll;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n_pad; j += stride) {
        bool ok = false;
        if (j < n) {
            const int64_t p = idx ? (int64_t)idx[j] : j;
            ok = p >= 0 && vg_valid(c, p);
            len[j] = ok ? (int32_t)load_view(c, p).len : 0;
        }
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, ok);
        if (lane == 0 && out_valid) out_valid[j >> 5] = m;
    }
}

// bytes of rows idx[j] (or j) to out + offs[j]; one warp per 32 rows, each
// string copied by the whole warp (coalesced for long strings)
__global__ void pack_kernel(VgCol c, const int32_t *idx, int64_t n, const int64_t *offs, char *out) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; w0 < n; w0 += warps * 32) {
        const int64_t j = w0 + lane;
        const char *src = nullptr;
        uint32_t len = 0;
        int64_t dst = 0;
        if (j < n) {
            const int64_t p = idx ? (int64_t)idx[j] : j;
            if (p >= 0 && vg_valid(c, p)) {
                const VgStrView v = load_view(c, p);
                src = v.ptr;
                len = v.len;
                dst = offs[j];
            }
        }
        for (int r = 0; r < 32; r++) {
            const uint32_t l = __shfl_sync(0xFFFFFFFFu, len, r);
            if (l == 0) continue;
            const char *s = (const char *)__shfl_sync(0xFFFFFFFFu, (unsigned long long)src, r);
            const int64_t d = __shfl_sync(0xFFFFFFFFu, (long long)dst, r);
            for (uint32_t k = lane; k < l; k += 32) out[d + k] = s[k];
        }
    }
}

// ---------------------------------------------------------------------
// dictionaries
// ---------------------------------------------------------------------

// valid rows, their bytes and the longest of them, over the logical rows
__global__ void dict_prepass_kernel(VgCol c, const int32_t *sel, int64_t n_logical, unsigned long long *ctr) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n_pad = (n_logical + 31) & ~31ll;
    unsigned long long rows = 0, bytes = 0;
    uint32_t mx = 0;
    for (int64_t li = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; li < n_pad; li += stride) {
        if (li < n_logical) {
            const int64_t p = sel ? (int64_t)sel[li] : li;
            if (vg_valid(c, p)) {
                const uint32_t l = load_view(c, p).len;
                rows++;
                bytes += l;
                mx = l > mx ? l : mx;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        rows += __shfl_down_sync(0xFFFFFFFFu, rows, o);
        bytes += __shfl_down_sync(0xFFFFFFFFu, bytes, o);
        const uint32_t m2 = __shfl_down_sync(0xFFFFFFFFu, mx, o);
        mx = m2 > mx ? m2 : mx;
    }
    if (lane == 0 && rows) {
        atomicAdd(ctr + VG_DICT_ROWS, rows);
        atomicAdd(ctr + VG_DICT_BYTES, bytes);
        atomicMax(ctr + VG_DICT_MAXLEN, (unsigned long long)mx);
    }
}

VG_DEV bool arena_equal(const char *a, const char *b, uint32_t len) {
    for (uint32_t k = 0; k < len; k++)
        if (__ldcg((const unsigned char *)a + k) != (unsigned char)b[k]) return false;
    return true;
}

// The code of string v: its entry if present, else (insert) a new entry
// with the next code and a copy of its bytes in the arena, else (no
// insert) -1.  The host has made room for every row of the launch, so
// neither the table (at most half full) nor the codes or the arena can run
// out; a slot another thread is filling is waited for, boundedly.
VG_DEV int64_t dict_code(const VgStrDict &d, const VgStrView &v, bool insert, uint32_t *err) {
    const uint64_t h = str_hash(v.ptr, v.len);
    const uint64_t mask = (uint64_t)d.cap - 1;
    uint64_t i = h & mask;
    for (int64_t probe = 0; probe < d.cap; probe++, i = (i + 1) & mask) {
        uint32_t s = *(volatile uint32_t *)(d.slot + i);
        for (;;) {                      // until the slot holds a code
            if (s == kEmpty) {
                if (!insert) return -1;
                const uint32_t old = atomicCAS(d.slot + i, kEmpty, kBusy);
                if (old != kEmpty) { s = old; continue; }
                const unsigned long long code = atomicAdd(d.ctr + VG_DICT_CODES, 1ull);
                const unsigned long long off = atomicAdd(d.ctr + VG_DICT_USED, (unsigned long long)v.len);
                if (code >= (unsigned long long)d.codes_cap || off + v.len > (unsigned long long)d.arena_cap) {
                    atomicOr(err, VG_ERR_FULL);     // the host made room for every row: cannot happen
                    atomicExch(d.slot + i, kEmpty);
                    return 0;
                }
                for (uint32_t k = 0; k < v.len; k++) d.arena[off + k] = v.ptr[k];
                atomicMax(d.ctr + VG_DICT_MAXLEN, (unsigned long long)v.len);
                d.c_hash[code] = h;
                d.c_off[code] = (int64_t)off;
                d.c_len[code] = v.len;
                __threadfence();
                atomicExch(d.slot + i, (uint32_t)code);
                return (int64_t)code;
            }
            if (s == kBusy) {
                s = vg_wait_while(d.slot + i, kBusy, s, VG_SPIN_LIMIT);
                if (s == kBusy) {
                    atomicOr(err, VG_ERR_WAIT);
                    return 0;
                }
                continue;
            }
            break;
        }
        if (__ldcg((const unsigned long long *)d.c_hash + s) == h && __ldcg(d.c_len + s) == v.len &&
            arena_equal(d.arena + __ldcg((const long long *)d.c_off + s), v.ptr, v.len))
            return (int64_t)s;
    }
    atomicOr(err, VG_ERR_FULL);
    return 0;
}

// codes[p] for the logical rows (p = sel[li] or li); NA rows get 0
__global__ void dict_encode_kernel(VgStrDict d, VgCol c, const int32_t *sel, int64_t n_logical, int insert,
                                   int64_t *codes, uint32_t *err) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t li = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; li < n_logical; li += stride) {
        const int64_t p = sel ? (int64_t)sel[li] : li;
        int64_t code = 0;
        if (vg_valid(c, p)) code = dict_code(d, load_view(c, p), insert != 0, err);
        codes[p] = code;
    }
}

// the slot table rebuilt from the codes' hashes (every code distinct)
__global__ void dict_rehash_kernel(VgStrDict d, int64_t n_codes, uint32_t *err) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const uint64_t mask = (uint64_t)d.cap - 1;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n_codes; c += stride) {
        uint64_t i = d.c_hash[c] & mask;
        int64_t probe = 0;
        for (; probe < d.cap; probe++, i = (i + 1) & mask)
            if (atomicCAS(d.slot + i, kEmpty, (uint32_t)c) == kEmpty) break;
        if (probe == d.cap) atomicOr(err, VG_ERR_FULL);
    }
}

// views of the strings of codes[j] (through map[] when given), NA where
// the validity bit of j is clear
__global__ void dict_views_kernel(VgStrDict d, const int64_t *codes, const uint32_t *valid, const int32_t *map,
                                  int64_t n, VgStrView *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        const bool ok = valid == nullptr || ((valid[j >> 5] >> (j & 31)) & 1u);
        VgStrView v;
        v.len = 0; v.pre = 0; v.ptr = d.arena;
        if (ok) {
            int64_t c = codes[j];
            if (map) c = map[c];
            v = vg_str_view(d.arena + d.c_off[c], d.c_len[c]);
        }
        out[j] = v;
    }
}

// order words of the codes' strings: column w (of n_chunks) holds bytes
// [8w, 8w + 8) big-endian, zero-padded, sign-flipped so that the signed
// order of the int64 is the bytes' order; the last column the length.
// Lexicographic order over these columns is memcmp order with the shorter
// string first on a common prefix.
__global__ void dict_chunks_kernel(VgStrDict d, int64_t n_codes, int n_chunks, int64_t *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n_codes; c += stride) {
        const unsigned char *s = (const unsigned char *)d.arena + d.c_off[c];
        const uint32_t len = d.c_len[c];
        const uint32_t last = len ? len - 1 : 0;
        for (int w = 0; w < n_chunks; w++) {
            uint64_t x = 0;
            for (int k = 0; k < 8; k++) {
                // every byte is read (at a clamped position inside the
                // string) and masked, rather than read conditionally
                const uint32_t at = (uint32_t)w * 8u + (uint32_t)k;
                const uint32_t b = len ? (uint32_t)s[at < last ? at : last] : 0u;
                const uint32_t m = at < len ? 0xFFu : 0u;
                x = (x << 8) | (uint64_t)(b & m);
            }
            out[(int64_t)w * n_codes + c] = (int64_t)(x ^ 0x8000000000000000ull);
        }
        out[(int64_t)n_chunks * n_codes + c] = (int64_t)len;
    }
}

__global__ void rank_kernel(const int32_t *perm, int64_t n, int64_t *rank) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) rank[perm[r]] = r;
}

// out[i] = table[codes[i]] where row i is valid (voff: bit offset of row 0)
__global__ void map_codes_kernel(const int64_t *table, const int64_t *codes, const uint32_t *valid, int voff,
                                 int64_t n, int64_t *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int64_t r = i + voff;
        const bool ok = valid == nullptr || ((valid[r >> 5] >> (r & 31)) & 1u);
        out[i] = ok ? table[codes[i]] : 0;
    }
}

// key word k of the listed group-table slots: code -> rank (NA keys kept)
__global__ void remap_keys_kernel(VgGroupTable gt, int k, const int32_t *slots, int64_t n, const int64_t *rank) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        const int64_t s = slots[j];
        if ((gt.nullmask[s] >> k) & 1u) continue;
        uint64_t *w = gt.keys + (int64_t)k * gt.cap + s;
        *w = (uint64_t)rank[*w];
    }
}

}  // namespace

extern "C" {

const char *vgk_str_last_error(void) { return g_err; }

int vgk_str_views(const int64_t *d_offs, int64_t base, const char *d_bytes, int64_t n, VgStrView *d_out,
                  vg_stream_t s) {
    if (n <= 0) return 0;
    views_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)s>>>(d_offs, base, d_bytes, n, d_out);
    vg_launch_counter++;
    return check(cudaGetLastError(), "string views");
}

int vgk_str_lengths(const VgCol *c, const int32_t *d_idx, int64_t n, int32_t *d_len, uint32_t *d_valid,
                    vg_stream_t s) {
    if (n <= 0) return 0;
    lengths_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)s>>>(*c, d_idx, n, d_len, d_valid);
    vg_launch_counter++;
    return check(cudaGetLastError(), "string lengths");
}

int vgk_str_pack(const VgCol *c, const int32_t *d_idx, int64_t n, const int64_t *d_offs, char *d_out,
                 vg_stream_t s) {
    if (n <= 0) return 0;
    pack_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)s>>>(*c, d_idx, n, d_offs, d_out);
    vg_launch_counter++;
    return check(cudaGetLastError(), "string pack");
}

int vgk_dict_prepass(const VgCol *c, const int32_t *d_sel, int64_t n_logical, unsigned long long *d_ctr,
                     vg_stream_t s) {
    if (n_logical <= 0) return 0;
    dict_prepass_kernel<<<grid_for(n_logical, 256), 256, 0, (cudaStream_t)s>>>(*c, d_sel, n_logical, d_ctr);
    vg_launch_counter++;
    return check(cudaGetLastError(), "string dictionary");
}

int vgk_dict_encode(const VgStrDict *d, const VgCol *c, const int32_t *d_sel, int64_t n_logical, int insert,
                    int64_t *d_codes, uint32_t *d_err, vg_stream_t s) {
    if (n_logical <= 0) return 0;
    dict_encode_kernel<<<grid_for(n_logical, 256), 256, 0, (cudaStream_t)s>>>(*d, *c, d_sel, n_logical, insert,
                                                                             d_codes, d_err);
    vg_launch_counter++;
    return check(cudaGetLastError(), "string dictionary encode");
}

int vgk_dict_rehash(const VgStrDict *d, int64_t n_codes, uint32_t *d_err, vg_stream_t s) {
    cudaStream_t st = (cudaStream_t)s;
    if (check(cudaMemsetAsync(d->slot, 0xFF, (size_t)d->cap * 4, st), "string dictionary rehash")) return -1;
    if (n_codes <= 0) return 0;
    dict_rehash_kernel<<<grid_for(n_codes, 256), 256, 0, st>>>(*d, n_codes, d_err);
    vg_launch_counter++;
    return check(cudaGetLastError(), "string dictionary rehash");
}

int vgk_dict_views(const VgStrDict *d, const int64_t *d_codes, const uint32_t *d_valid, const int32_t *d_map,
                   int64_t n, VgStrView *d_out, vg_stream_t s) {
    if (n <= 0) return 0;
    dict_views_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)s>>>(*d, d_codes, d_valid, d_map, n, d_out);
    vg_launch_counter++;
    return check(cudaGetLastError(), "string dictionary views");
}

int vgk_dict_chunks(const VgStrDict *d, int64_t n_codes, int n_chunks, int64_t *d_out, vg_stream_t s) {
    if (n_codes <= 0) return 0;
    dict_chunks_kernel<<<grid_for(n_codes, 256), 256, 0, (cudaStream_t)s>>>(*d, n_codes, n_chunks, d_out);
    vg_launch_counter++;
    return check(cudaGetLastError(), "string dictionary order");
}

int vgk_rank_of(const int32_t *d_perm, int64_t n, int64_t *d_rank, vg_stream_t s) {
    if (n <= 0) return 0;
    rank_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)s>>>(d_perm, n, d_rank);
    vg_launch_counter++;
    return check(cudaGetLastError(), "string dictionary order");
}

int vgk_map_codes(const int64_t *d_table, const int64_t *d_codes, const uint32_t *d_valid, int voff, int64_t n,
                  int64_t *d_out, vg_stream_t s) {
    if (n <= 0) return 0;
    map_codes_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)s>>>(d_table, d_codes, d_valid, voff, n, d_out);
    vg_launch_counter++;
    return check(cudaGetLastError(), "string order");
}

int vgk_group_keys_remap(const VgGroupTable *gt, int k, const int32_t *d_slots, int64_t n, const int64_t *d_rank,
                         vg_stream_t s) {
    if (n <= 0) return 0;
    remap_keys_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)s>>>(*gt, k, d_slots, n, d_rank);
    vg_launch_counter++;
    return check(cudaGetLastError(), "group key order");
}

}  // extern "C"
