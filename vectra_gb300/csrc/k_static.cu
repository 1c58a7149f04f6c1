// k_static.cu -- fixed device scratch for vgpu_filter_select_static.
//
// The allocation-free filter entry point carves its working space (the
// predicate arguments, one keep word per 32 rows, per-block counts, the
// selected-row total and an error word) out of this file-scope array
// instead of allocating it.  Its address is looked up once per device with
// cudaGetSymbolAddress and cached; that first lookup is the only set-up.
// The selection it computes is filter_next_batch's (src/filter.c:13-64).

#include <cstdio>
#include "vgpu_internal.h"

constexpr size_t VG_STATIC_SCRATCH_BYTES = ((size_t)1 << 20) + ((size_t)1 << 16);   // 1 MiB + 64 KiB

namespace {

__device__ __align__(256) unsigned char g_static_scratch[VG_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
void *g_addr[kMaxDevices];
char g_msg[256];

}  // namespace

extern "C" {

// Address and size of this device's static scratch; -1 (message in
// vgk_static_scratch_error) if the device cannot be queried.
int vgk_static_scratch(void **ptr, size_t *bytes) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        snprintf(g_msg, sizeof(g_msg), "static scratch: cudaGetDevice: %s", cudaGetErrorString(e));
        return -1;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        snprintf(g_msg, sizeof(g_msg), "static scratch: device %d out of range", dev);
        return -1;
    }
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) {
            snprintf(g_msg, sizeof(g_msg), "static scratch: cudaGetSymbolAddress: %s",
                     cudaGetErrorString(e));
            return -1;
        }
        g_addr[dev] = p;
    }
    *ptr = g_addr[dev];
    *bytes = VG_STATIC_SCRATCH_BYTES;
    return 0;
}

const char *vgk_static_scratch_error(void) { return g_msg; }

}  // extern "C"
