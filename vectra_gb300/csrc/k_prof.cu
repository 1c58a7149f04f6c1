// k_prof.cu -- optional per-kernel timing with CUDA events recorded on the
// launching stream (off by default; the benchmark turns it on to report the
// dominant kernel's duration next to its algorithmic bytes).

#include <cstdio>
#include <vector>
#include "k_common.cuh"

namespace {
struct Pair { int cls; cudaEvent_t a, b; };
bool g_on = false;
std::vector<Pair> g_pending;
double g_ms[VG_PROF_CLASSES];
unsigned long long g_n[VG_PROF_CLASSES];
cudaEvent_t g_open[VG_PROF_CLASSES];

void resolve() {
    for (auto &p : g_pending) {
        cudaEventSynchronize(p.b);
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            g_ms[p.cls] += ms;
            g_n[p.cls] += 1;
        }
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    g_pending.clear();
}
}  // namespace

void vg_prof_begin(int cls, cudaStream_t s) {
    if (!g_on || cls < 0 || cls >= VG_PROF_CLASSES) return;
    cudaEventCreate(&g_open[cls]);
    cudaEventRecord(g_open[cls], s);
}

void vg_prof_end(int cls, cudaStream_t s) {
    if (!g_on || cls < 0 || cls >= VG_PROF_CLASSES || !g_open[cls]) return;
    Pair p;
    p.cls = cls;
    p.a = g_open[cls];
    cudaEventCreate(&p.b);
    cudaEventRecord(p.b, s);
    g_pending.push_back(p);
    g_open[cls] = nullptr;
}

extern "C" {

void vgpu_profile_enable(int on) {
    resolve();
    g_on = on != 0;
}

void vgpu_profile_reset(void) {
    resolve();
    for (int i = 0; i < VG_PROF_CLASSES; i++) { g_ms[i] = 0; g_n[i] = 0; }
}

// profiling on for a while (the partitioned path's fan-out tuning times
// its launches with it): the previous state, to restore
int vg_prof_force_on(void) {
    resolve();
    const int prev = g_on ? 1 : 0;
    g_on = true;
    return prev;
}

void vg_prof_restore(int prev) {
    resolve();
    g_on = prev != 0;
}

// total milliseconds and launches of a kernel class since the last reset
double vgpu_profile_ms(int cls, unsigned long long *launches) {
    resolve();
    if (cls < 0 || cls >= VG_PROF_CLASSES) return 0.0;
    if (launches) *launches = g_n[cls];
    return g_ms[cls];
}

}  // extern "C"
