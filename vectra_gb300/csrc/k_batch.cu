// k_batch.cu -- many small independent queries (a query set) in a few
// persistent launches captured once into a CUDA graph (vgpu_queryset_*).
//
// Two query kinds, the shapes of the reference's group-agg and hash-join
// nodes on one key column (src/group_agg.c:155-281, src/join.c:156-480):
//   GROUP  group_by(key) |> summarise(sum(value), mean(value), n())
//          (exact double sums: correctly rounded, as the node path)
//   JOIN   inner_join(probe, build, key) over unique build keys: the
//          (probe row, build row) pairs in probe row order
// Instances are cut into work items of at most kChunk rows; persistent
// CTAs (one per SM) take items from atomic counters:
//   phase 0  empty every instance's table
//   phase 1  group chunks aggregate into their instance's table; join
//            build chunks insert their keys
//   phase 2  group instances write their groups (table order); join probe
//            chunks count their matches
//   phase 3  join probe chunks write their pairs at the offset the
//            instance's earlier chunks leave (probe order)
// Every instance's table lives in one scratch block sized at prepare time;
// small tables stay in L2 while their instance runs.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>
#include "k_set_dev.cuh"

#include "vgpu.h"

namespace {

constexpr int kSetThreads = 512;
constexpr int64_t kChunk = 65536;

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
};

// ---------------------------------------------------------------------
// phase 0: empty the tables
// ---------------------------------------------------------------------
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
            for (int64_t s = W.lo + threadIdx.x; s < W.hi; s += blockDim.x) {
                const GSlot &g = t[s];
                if (g.cnt == 0) continue;
                const unsigned long long o = atomicAdd((unsigned long long *)I.q.out_rows, 1ull);
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

int64_t pow2_at_least(int64_t x) {
    int64_t c = 64;
    while (c < x) c <<= 1;
    return c;
}

}  // namespace

extern "C" {

void vg_set_error(const char *fmt, ...);
void vgpu_queryset_free(void *plan);

static int queryset_prepare(const VgpuSetQuery *qs, int n, void **plan_out) {
    *plan_out = nullptr;
    if (n <= 0 || !qs) { snprintf(g_err, sizeof(g_err), "vgpu_queryset_prepare: no queries"); return -1; }
    Plan *P = new Plan();
    memset(P, 0, sizeof(*P));
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
            I.cap = pow2_at_least(2 * (q.max_groups < q.n ? q.max_groups : (q.n > 0 ? q.n : 1)));
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
            I.cap = pow2_at_least(2 * (q.n_build > 0 ? q.n_build : 1));
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
    P->grid = sms > 0 ? sms * (2048 / kSetThreads) : 64;
    if (ck(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "batch capture")) { vgpu_queryset_free(P); return -1; }
    cudaMemsetAsync(P->d_ctr, 0, 32, st);
    set_init_kernel<<<P->grid, kSetThreads, 0, st>>>(P->d_inst, n);
    set_phase1_kernel<<<P->grid, kSetThreads, 0, st>>>(P->d_inst, P->d_items1, P->n1, P->d_ctr);
    set_phase2_kernel<<<P->grid, kSetThreads, 0, st>>>(P->d_inst, P->d_items2, P->n2, P->d_chunk_cnt, P->d_ctr);
    set_phase3_kernel<<<P->grid, kSetThreads, 0, st>>>(P->d_inst, P->d_items3, P->n3, P->d_chunk_cnt, P->d_ctr);
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

int vgpu_queryset_prepare(const VgpuSetQuery *qs, int n, void **plan) {
    g_err[0] = 0;
    const int rc = queryset_prepare(qs, n, plan);
    if (rc) vg_set_error("%s", g_err);
    return rc;
}

int vgpu_queryset_run(void *plan) {
    g_err[0] = 0;
    const int rc = queryset_run(plan);
    if (rc) vg_set_error("%s", g_err);
    return rc;
}

}  // extern "C"
