// k_batch.cu -- many small independent queries (a query set) in a few
// persistent launches captured once into a CUDA graph (vgpu_queryset_*).
//
// Two query kinds, the shapes of the reference's group-agg and hash-join
// nodes on one key column (src/group_agg.c:155-281, src/join.c:156-480):
//   GROUP  group_by(key) |> summarise(sum(value), mean(value), n())
//          (exact double sums: correctly rounded, as the node path)
//   JOIN   inner_join(probe, build, key) over unique build keys: the
//          (probe row, build row) pairs in probe row order
// Instances are cut into work items of at most `chunk` rows; persistent
// CTAs take items from atomic counters:
//   phase 0  empty every instance's table
//   phase 1  group chunks aggregate into their instance's table; join
//            build chunks insert their keys
//   phase 2  group instances write their groups (table order); join probe
//            chunks count their matches
//   phase 3  join probe chunks write their pairs at the offset the
//            instance's earlier chunks leave (probe order)
// Every instance's table lives in one scratch block sized at prepare time;
// small tables stay in L2 while their instance runs.  Threads per CTA,
// rows per work item and the tables' load factor are chosen per set shape
// by vgpu_queryset_tune (measured on the set) and recorded.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>
#include "k_set_dev.cuh"

#include "vgpu.h"

namespace {

// Launch parameters of a query set; the defaults, or what
// vgpu_queryset_tune measured fastest for sets of the same shape.
struct Cfg {
    int threads = 512;            // per CTA: 256, 512 or 1024
    int64_t chunk = 65536;        // rows per work item (each instance's fan-out)
    int cap_mult = 2;             // table capacity >= cap_mult x keys (load <= 1/cap_mult)
};

int ck(cudaError_t e, const char *what) { return check(e, what); }

struct Inst {                 // a query with its scratch
    VgpuSetQuery q;
    int64_t cap;              // power of two; slot cap is the marker key's
    void *table;              // GSlot[cap + 1] or JSlot[cap + 1]
    int64_t first_chunk;      // index of the instance's first probe chunk (join)
};

struct Item {
    int32_t inst;
    int32_t chunk;            // index within the instance
    int64_t lo, hi;           // rows [lo, hi)
};

struct Plan {
    int n_inst;
    Inst *d_inst;
    Item *d_items1, *d_items2, *d_items3;   // phases 1..3 work lists
    int n1, n2, n3;
    int64_t *d_chunk_cnt;     // matches per join probe chunk
    uint32_t *d_ctr;          // [0..3] phase counters, [4] error bits
    void *block;              // all tables
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    cudaStream_t stream;
    int grid;
    Cfg cfg;
};

// ---------------------------------------------------------------------
// phase 0: empty the tables
// ---------------------------------------------------------------------
template <int kSetThreads>
__global__ void __launch_bounds__(kSetThreads) set_init_kernel(const Inst *inst, int n_inst) {
    for (int i = blockIdx.x; i < n_inst; i += gridDim.x) {
        const Inst &I = inst[i];
        if (I.q.kind == VGPU_SET_GROUP) {
            GSlot *t = (GSlot *)I.table;
            for (int64_t s = threadIdx.x; s <= I.cap; s += blockDim.x) {
                GSlot &g = t[s];
                g.key = kEmpty;
                g.cnt = 0;
                g.base = kBaseUnset;
                g.flags = 0;
#pragma unroll
                for (int w = 0; w < kWin; w++) g.win[w] = 0;
                g.fs = 0.0;
                g.fc = 0.0;
            }
        } else {
            JSlot *t = (JSlot *)I.table;
            for (int64_t s = threadIdx.x; s <= I.cap; s += blockDim.x) {
                t[s].key = kEmpty;
                t[s].row = -1;
            }
        }
        if (I.q.out_rows && threadIdx.x == 0) *I.q.out_rows = 0;
    }
}

// ---------------------------------------------------------------------
// phase 1: aggregate / build
// ---------------------------------------------------------------------
template <int kSetThreads>
__global__ void __launch_bounds__(kSetThreads) set_phase1_kernel(const Inst *inst, const Item *items, int n_items,
                                                                uint32_t *ctr) {
    __shared__ int item;
    for (;;) {
        if (threadIdx.x == 0) item = (int)atomicAdd(ctr + 1, 1u);
        __syncthreads();
        const int it = item;
        __syncthreads();
        if (it >= n_items) return;
        const Item W = items[it];
        const Inst &I = inst[W.inst];
        if (I.q.kind == VGPU_SET_GROUP) {
            GSlot *t = (GSlot *)I.table;
            for (int64_t r = W.lo + threadIdx.x; r < W.hi; r += blockDim.x) {
                const uint64_t k = (uint64_t)__ldg((const long long *)I.q.key + r);
                const int64_t s = g_slot(t, I.cap, k);
                if (s < 0) { atomicOr(ctr + 4, VG_ERR_FULL); continue; }
                atomicAdd(&t[s].cnt, 1ull);
                g_add(t[s], (uint64_t)__ldg((const long long *)I.q.value + r));
            }
        } else {
            JSlot *t = (JSlot *)I.table;
            for (int64_t r = W.lo + threadIdx.x; r < W.hi; r += blockDim.x) {
                const uint64_t k = (uint64_t)__ldg((const long long *)I.q.build_key + r);
                const int64_t s = j_insert(t, I.cap, k);
                if (s < 0) { atomicOr(ctr + 4, VG_ERR_FULL); continue; }
                // a repeated build key: the later row wins the slot, and the
                // duplicate is reported (the batched join takes unique keys)
                if (atomicExch((unsigned long long *)&t[s].row, (unsigned long long)r) != ~0ull)
                    atomicOr(ctr + 4, VG_ERR_PROG);
            }
        }
    }
}

// ---------------------------------------------------------------------
// phase 2: group results / join match counts
// ---------------------------------------------------------------------
template <int kSetThreads>
__global__ void __launch_bounds__(kSetThreads) set_phase2_kernel(const Inst *inst, const Item *items, int n_items,
                                                                int64_t *chunk_cnt, uint32_t *ctr) {
    __shared__ int item;
    __shared__ unsigned long long s_cnt;
    for (;;) {
        if (threadIdx.x == 0) { item = (int)atomicAdd(ctr + 2, 1u); s_cnt = 0; }
        __syncthreads();
        const int it = item;
        if (it >= n_items) return;
        const Item W = items[it];
        const Inst &I = inst[W.inst];
        if (I.q.kind == VGPU_SET_GROUP) {
            // slots [lo, hi) of the table (items cover cap + 1 slots)
            const GSlot *t = (const GSlot *)I.table;
            const int lane = threadIdx.x & 31;
            // output rows taken per warp (one counter update per 32 slots)
            for (int64_t s0 = W.lo; s0 < W.hi; s0 += blockDim.x) {
                const int64_t s = s0 + threadIdx.x;
                const bool has = s < W.hi && t[s].cnt != 0;
                const unsigned m = __ballot_sync(0xFFFFFFFFu, has);
                unsigned long long ob = 0;
                if (lane == 0 && m) ob = atomicAdd((unsigned long long *)I.q.out_rows, (unsigned long long)__popc(m));
                ob = __shfl_sync(0xFFFFFFFFu, ob, 0);
                if (!has) continue;
                const GSlot &g = t[s];
                const unsigned long long o = ob + (unsigned long long)__popc(m & ((1u << lane) - 1u));
                if ((int64_t)o >= I.q.max_groups) { atomicOr(ctr + 4, VG_ERR_FULL); continue; }
                const double sum = g_sum(g);
                I.q.out_key[o] = (int64_t)g.key;
                I.q.out_sum[o] = sum;
                I.q.out_mean[o] = __ddiv_rn(sum, (double)g.cnt);
                I.q.out_n[o] = (int64_t)g.cnt;
            }
        } else {
            const JSlot *t = (const JSlot *)I.table;
            unsigned long long c = 0;
            for (int64_t r = W.lo + threadIdx.x; r < W.hi; r += blockDim.x)
                if (j_find(t, I.cap, (uint64_t)__ldg((const long long *)I.q.key + r)) >= 0) c++;
            c = __reduce_add_sync(0xFFFFFFFFu, (unsigned)c);
            if ((threadIdx.x & 31) == 0 && c) atomicAdd(&s_cnt, c);
            __syncthreads();
            if (threadIdx.x == 0) {
                chunk_cnt[I.first_chunk + W.chunk] = (int64_t)s_cnt;
                atomicAdd((unsigned long long *)I.q.out_rows, s_cnt);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------
// phase 3: join pairs in probe order
// ---------------------------------------------------------------------
template <int kSetThreads>
__global__ void __launch_bounds__(kSetThreads) set_phase3_kernel(const Inst *inst, const Item *items, int n_items,
                                                                const int64_t *chunk_cnt, uint32_t *ctr) {
    __shared__ int item;
    __shared__ int64_t s_base;
    __shared__ int warp_tot[kSetThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (;;) {
        if (threadIdx.x == 0) item = (int)atomicAdd(ctr + 3, 1u);
        __syncthreads();
        const int it = item;
        if (it >= n_items) return;
        const Item W = items[it];
        const Inst &I = inst[W.inst];
        if (threadIdx.x == 0) {
            int64_t b = 0;
            for (int c = 0; c < W.chunk; c++) b += chunk_cnt[I.first_chunk + c];
            s_base = b;
        }
        __syncthreads();
        const JSlot *t = (const JSlot *)I.table;
        for (int64_t r0 = W.lo; r0 < W.hi; r0 += blockDim.x) {
            const int64_t r = r0 + threadIdx.x;
            long long br = -1;
            if (r < W.hi) br = j_find(t, I.cap, (uint64_t)__ldg((const long long *)I.q.key + r));
            const unsigned m = __ballot_sync(0xFFFFFFFFu, br >= 0);
            if (lane == 0) warp_tot[wid] = __popc(m);
            __syncthreads();
            int before = 0, total = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
                if (w < wid) before += warp_tot[w];
                total += warp_tot[w];
            }
            if (br >= 0) {
                const int64_t o = s_base + before + __popc(m & ((1u << lane) - 1u));
                I.q.out_probe[o] = (int32_t)r;
                I.q.out_build[o] = (int32_t)br;
            }
            __syncthreads();
            if (threadIdx.x == 0) s_base += total;
            __syncthreads();
        }
    }
}

// the four phases of a run, as captured into the set's graph
template <int T>
void capture_phases(Plan *P, int n, cudaStream_t st) {
    set_init_kernel<T><<<P->grid, T, 0, st>>>(P->d_inst, n);
    set_phase1_kernel<T><<<P->grid, T, 0, st>>>(P->d_inst, P->d_items1, P->n1, P->d_ctr);
    set_phase2_kernel<T><<<P->grid, T, 0, st>>>(P->d_inst, P->d_items2, P->n2, P->d_chunk_cnt, P->d_ctr);
    set_phase3_kernel<T><<<P->grid, T, 0, st>>>(P->d_inst, P->d_items3, P->n3, P->d_chunk_cnt, P->d_ctr);
}

int64_t pow2_at_least(int64_t x) {
    int64_t c = 64;
    while (c < x) c <<= 1;
    return c;
}

}  // namespace

extern "C" {

void vg_set_error(const char *fmt, ...);
void vgpu_queryset_free(void *plan);

static int queryset_prepare(const VgpuSetQuery *qs, int n, const Cfg &cfg, void **plan_out) {
    const int64_t kChunk = cfg.chunk;
    *plan_out = nullptr;
    if (n <= 0 || !qs) { snprintf(g_err, sizeof(g_err), "vgpu_queryset_prepare: no queries"); return -1; }
    Plan *P = new Plan();      // value-initialised: every pointer and count zero
    P->n_inst = n;
    std::vector<Inst> inst((size_t)n);
    std::vector<Item> it1, it2, it3;
    size_t bytes = 0;
    int64_t chunks = 0;
    for (int i = 0; i < n; i++) {
        const VgpuSetQuery &q = qs[i];
        Inst &I = inst[(size_t)i];
        memset(&I, 0, sizeof(I));
        I.q = q;
        if (q.kind == VGPU_SET_GROUP) {
            if (q.n < 0 || q.max_groups <= 0 || !q.out_rows || (q.n > 0 && (!q.key || !q.value))) {
                snprintf(g_err, sizeof(g_err), "vgpu_queryset_prepare: query %d: bad group arguments", i);
                delete P;
                return -1;
            }
            I.cap = pow2_at_least(cfg.cap_mult * (q.max_groups < q.n ? q.max_groups : (q.n > 0 ? q.n : 1)));
            bytes += (size_t)(I.cap + 1) * sizeof(GSlot);
            for (int64_t lo = 0, c = 0; lo < q.n; lo += kChunk, c++)
                it1.push_back(Item{i, (int32_t)c, lo, lo + kChunk < q.n ? lo + kChunk : q.n});
            for (int64_t lo = 0; lo <= I.cap; lo += kChunk)
                it2.push_back(Item{i, 0, lo, lo + kChunk < I.cap + 1 ? lo + kChunk : I.cap + 1});
        } else if (q.kind == VGPU_SET_JOIN) {
            if (q.n < 0 || q.n_build < 0 || !q.out_rows || (q.n > 0 && !q.key) || (q.n_build > 0 && !q.build_key) ||
                q.n >= ((int64_t)1 << 31) || q.n_build >= ((int64_t)1 << 31)) {
                snprintf(g_err, sizeof(g_err), "vgpu_queryset_prepare: query %d: bad join arguments", i);
                delete P;
                return -1;
            }
            I.cap = pow2_at_least(cfg.cap_mult * (q.n_build > 0 ? q.n_build : 1));
            bytes += (size_t)(I.cap + 1) * sizeof(JSlot);
            for (int64_t lo = 0, c = 0; lo < q.n_build; lo += kChunk, c++)
                it1.push_back(Item{i, (int32_t)c, lo, lo + kChunk < q.n_build ? lo + kChunk : q.n_build});
            I.first_chunk = chunks;
            for (int64_t lo = 0, c = 0; lo < q.n; lo += kChunk, c++) {
                it2.push_back(Item{i, (int32_t)c, lo, lo + kChunk < q.n ? lo + kChunk : q.n});
                it3.push_back(Item{i, (int32_t)c, lo, lo + kChunk < q.n ? lo + kChunk : q.n});
                chunks++;
            }
        } else {
            snprintf(g_err, sizeof(g_err), "vgpu_queryset_prepare: query %d: unknown kind %d", i, q.kind);
            delete P;
            return -1;
        }
        bytes = (bytes + 255) & ~(size_t)255;
    }
    // large work items first: the persistent CTAs finish together
    auto by_size = [](const Item &a, const Item &b) { return (a.hi - a.lo) > (b.hi - b.lo); };
    std::stable_sort(it1.begin(), it1.end(), by_size);
    std::stable_sort(it2.begin(), it2.end(), by_size);
    if (ck(cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking), "batch stream")) { delete P; return -1; }
    char *blk = nullptr;
    size_t meta = ((sizeof(Inst) * (size_t)n + 255) & ~(size_t)255) +
                  ((sizeof(Item) * (it1.size() + it2.size() + it3.size() + 3) + 255) & ~(size_t)255) +
                  ((sizeof(int64_t) * (size_t)(chunks + 1) + 255) & ~(size_t)255) + 256;
    if (ck(cudaMalloc(&blk, bytes + meta), "batch scratch")) { cudaStreamDestroy(P->stream); delete P; return -1; }
    P->block = blk;
    size_t o = 0;
    for (int i = 0; i < n; i++) {
        Inst &I = inst[(size_t)i];
        I.table = blk + o;
        o += (size_t)(I.cap + 1) * (I.q.kind == VGPU_SET_GROUP ? sizeof(GSlot) : sizeof(JSlot));
        o = (o + 255) & ~(size_t)255;
    }
    P->d_inst = (Inst *)(blk + o);
    o += (sizeof(Inst) * (size_t)n + 255) & ~(size_t)255;
    P->d_items1 = (Item *)(blk + o);
    P->d_items2 = P->d_items1 + it1.size();
    P->d_items3 = P->d_items2 + it2.size();
    o += (sizeof(Item) * (it1.size() + it2.size() + it3.size() + 3) + 255) & ~(size_t)255;
    P->d_chunk_cnt = (int64_t *)(blk + o);
    o += (sizeof(int64_t) * (size_t)(chunks + 1) + 255) & ~(size_t)255;
    P->d_ctr = (uint32_t *)(blk + o);
    P->n1 = (int)it1.size();
    P->n2 = (int)it2.size();
    P->n3 = (int)it3.size();
    cudaStream_t st = P->stream;
    cudaMemcpyAsync(P->d_inst, inst.data(), sizeof(Inst) * (size_t)n, cudaMemcpyHostToDevice, st);
    if (!it1.empty()) cudaMemcpyAsync(P->d_items1, it1.data(), sizeof(Item) * it1.size(), cudaMemcpyHostToDevice, st);
    if (!it2.empty()) cudaMemcpyAsync(P->d_items2, it2.data(), sizeof(Item) * it2.size(), cudaMemcpyHostToDevice, st);
    if (!it3.empty()) cudaMemcpyAsync(P->d_items3, it3.data(), sizeof(Item) * it3.size(), cudaMemcpyHostToDevice, st);
    if (ck(cudaStreamSynchronize(st), "batch prepare")) { vgpu_queryset_free(P); return -1; }
    // the whole run as one graph: reset the counters, the four phases
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    P->grid = sms > 0 ? sms * (2048 / cfg.threads) : 64;
    P->cfg = cfg;
    if (ck(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "batch capture")) { vgpu_queryset_free(P); return -1; }
    cudaMemsetAsync(P->d_ctr, 0, 32, st);
    if (cfg.threads == 256) capture_phases<256>(P, n, st);
    else if (cfg.threads == 1024) capture_phases<1024>(P, n, st);
    else capture_phases<512>(P, n, st);
    cudaError_t e = cudaStreamEndCapture(st, &P->graph);
    if (ck(e, "batch capture end") || ck(cudaGraphInstantiate(&P->exec, P->graph, 0), "batch graph")) {
        vgpu_queryset_free(P);
        return -1;
    }
    *plan_out = P;
    return 0;
}

static int queryset_run(void *plan) {
    Plan *P = (Plan *)plan;
    if (!P) { snprintf(g_err, sizeof(g_err), "vgpu_queryset_run: no plan"); return -1; }
    if (ck(cudaGraphLaunch(P->exec, P->stream), "batch launch")) return -1;
    vg_launch_counter += 4;
    uint32_t err = 0;
    cudaMemcpyAsync(&err, P->d_ctr + 4, 4, cudaMemcpyDeviceToHost, P->stream);
    if (ck(cudaStreamSynchronize(P->stream), "batch run")) return -1;
    if (err & VG_ERR_FULL) { snprintf(g_err, sizeof(g_err), "vgpu_queryset_run: a table or an output was too small"); return -1; }
    if (err & VG_ERR_PROG) { snprintf(g_err, sizeof(g_err), "vgpu_queryset_run: a join's build keys repeat"); return -1; }
    return 0;
}

void vgpu_queryset_free(void *plan) {
    Plan *P = (Plan *)plan;
    if (!P) return;
    if (P->exec) cudaGraphExecDestroy(P->exec);
    if (P->graph) cudaGraphDestroy(P->graph);
    if (P->block) cudaFree(P->block);
    if (P->stream) cudaStreamDestroy(P->stream);
    delete P;
}

}  // extern "C"

// ---------------------------------------------------------------------
// autotuning: launch parameters measured per query-set shape
// ---------------------------------------------------------------------
namespace {

struct Tuned {
    Cfg cfg;
    double ms;
    int candidates;
};

std::mutex g_tune_mu;
std::map<std::string, Tuned> g_tuned;
bool g_tune_loaded = false;

int lg2(double x) { return x < 1.0 ? 0 : (int)std::floor(std::log2(x)); }

// Shape of a set: how many group and join instances, total and largest
// instance rows, mean group cardinality -- each as a power of two.
std::string shape_of(const VgpuSetQuery *qs, int n) {
    int64_t ng = 0, nj = 0, rows = 0, maxr = 0;
    double card = 0.0;
    for (int i = 0; i < n; i++) {
        const VgpuSetQuery &q = qs[i];
        const int64_t r = q.n + (q.kind == VGPU_SET_JOIN ? q.n_build : 0);
        rows += r;
        maxr = r > maxr ? r : maxr;
        if (q.kind == VGPU_SET_GROUP) {
            ng++;
            card += (double)(q.max_groups < q.n ? q.max_groups : (q.n > 0 ? q.n : 1));
        } else {
            nj++;
        }
    }
    char buf[96];
    snprintf(buf, sizeof(buf), "g%d.j%d.r%d.m%d.c%d", lg2((double)ng), lg2((double)nj), lg2((double)rows),
             lg2((double)maxr), ng ? lg2(card / (double)ng) : 0);
    return buf;
}

// Recorded tunings persist in the file named by VGPU_TUNE_FILE (one line
// per measurement: shape threads chunk_rows table_mult ms candidates;
// the last line of a shape wins).
void load_tunings() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char *path = getenv("VGPU_TUNE_FILE");
    if (!path || !*path) return;
    FILE *f = fopen(path, "r");
    if (!f) return;
    char shape[96];
    Tuned t;
    long long chunk = 0;
    while (fscanf(f, "%95s %d %lld %d %lf %d", shape, &t.cfg.threads, &chunk, &t.cfg.cap_mult, &t.ms, &t.candidates) ==
           6) {
        t.cfg.chunk = chunk;
        if ((t.cfg.threads == 256 || t.cfg.threads == 512 || t.cfg.threads == 1024) && chunk >= 1024 &&
            (t.cfg.cap_mult == 2 || t.cfg.cap_mult == 4))
            g_tuned[shape] = t;
    }
    fclose(f);
}

void save_tuning(const std::string &shape, const Tuned &t) {
    const char *path = getenv("VGPU_TUNE_FILE");
    if (!path || !*path) return;
    FILE *f = fopen(path, "a");
    if (!f) return;
    fprintf(f, "%s %d %lld %d %.6f %d\n", shape.c_str(), t.cfg.threads, (long long)t.cfg.chunk, t.cfg.cap_mult, t.ms,
            t.candidates);
    fclose(f);
}

Cfg config_for(const VgpuSetQuery *qs, int n, bool *tuned) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    load_tunings();
    auto it = g_tuned.find(shape_of(qs, n));
    *tuned = it != g_tuned.end();
    return *tuned ? it->second.cfg : Cfg();
}

void fill(VgpuSetTuning *out, const std::string &shape, const Cfg &c, double ms, int candidates) {
    if (!out) return;
    memset(out, 0, sizeof(*out));
    out->threads = c.threads;
    out->table_mult = c.cap_mult;
    out->chunk_rows = c.chunk;
    out->ms = ms;
    out->candidates = candidates;
    snprintf(out->shape, sizeof(out->shape), "%s", shape.c_str());
}

// one run of a prepared plan, in milliseconds of wall time (the run waits)
double time_run(void *plan) {
    const auto t0 = std::chrono::steady_clock::now();
    if (queryset_run(plan) != 0) return -1.0;
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" {

int vgpu_queryset_prepare(const VgpuSetQuery *qs, int n, void **plan) {
    g_err[0] = 0;
    bool tuned = false;
    const Cfg cfg = (qs && n > 0) ? config_for(qs, n, &tuned) : Cfg();
    const int rc = queryset_prepare(qs, n, cfg, plan);
    if (rc) vg_set_error("%s", g_err);
    return rc;
}

int vgpu_queryset_prepare_with(const VgpuSetQuery *qs, int n, const VgpuSetTuning *params, void **plan) {
    g_err[0] = 0;
    Cfg cfg;
    if (params) {
        if ((params->threads != 256 && params->threads != 512 && params->threads != 1024) ||
            params->chunk_rows < 1024 || (params->table_mult != 2 && params->table_mult != 4)) {
            vg_set_error("vgpu_queryset_prepare_with: threads 256/512/1024, chunk_rows >= 1024, table_mult 2 or 4");
            return -1;
        }
        cfg.threads = params->threads;
        cfg.chunk = params->chunk_rows;
        cfg.cap_mult = params->table_mult;
    }
    const int rc = queryset_prepare(qs, n, cfg, plan);
    if (rc) vg_set_error("%s", g_err);
    return rc;
}

int vgpu_queryset_tuning(const VgpuSetQuery *qs, int n, VgpuSetTuning *out) {
    if (!qs || n <= 0) return 0;
    const std::string shape = shape_of(qs, n);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    load_tunings();
    auto it = g_tuned.find(shape);
    if (it == g_tuned.end()) {
        fill(out, shape, Cfg(), 0.0, 0);
        return 0;
    }
    fill(out, shape, it->second.cfg, it->second.ms, it->second.candidates);
    return 1;
}

// Times every candidate configuration on the set itself (one warm-up run
// and the best of `reps` timed runs each; the queries' outputs are simply
// rewritten) and records the fastest for the set's shape.
int vgpu_queryset_tune(const VgpuSetQuery *qs, int n, int reps, VgpuSetTuning *out) {
    g_err[0] = 0;
    if (!qs || n <= 0) {
        vg_set_error("vgpu_queryset_tune: no queries");
        return -1;
    }
    if (reps < 1) reps = 1;
    const int threads[] = {256, 512, 1024};
    const int64_t chunks[] = {16384, 65536, 262144};
    const int mults[] = {2, 4};
    Tuned best;
    best.ms = -1.0;
    best.candidates = 0;
    for (int t : threads)
        for (int64_t c : chunks)
            for (int m : mults) {
                Cfg cfg;
                cfg.threads = t;
                cfg.chunk = c;
                cfg.cap_mult = m;
                void *plan = nullptr;
                if (queryset_prepare(qs, n, cfg, &plan) != 0) continue;
                double ms = time_run(plan);        // warm-up (and a check that it runs)
                for (int r = 0; r < reps && ms >= 0.0; r++) {
                    const double x = time_run(plan);
                    ms = (r == 0 || x < ms) ? x : ms;
                }
                vgpu_queryset_free(plan);
                if (ms < 0.0) continue;
                best.candidates++;
                if (best.ms < 0.0 || ms < best.ms) {
                    best.cfg = cfg;
                    best.ms = ms;
                }
            }
    if (best.ms < 0.0) {
        vg_set_error("vgpu_queryset_tune: no configuration ran (%s)", g_err);
        return -1;
    }
    const std::string shape = shape_of(qs, n);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        load_tunings();
        g_tuned[shape] = best;
        save_tuning(shape, best);
    }
    fill(out, shape, best.cfg, best.ms, best.candidates);
    return 0;
}

int vgpu_queryset_run(void *plan) {
    g_err[0] = 0;
    const int rc = queryset_run(plan);
    if (rc) vg_set_error("%s", g_err);
    return rc;
}

}  // extern "C"
