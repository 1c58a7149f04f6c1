// jit_agg.cu -- run-time specialisation of the fused aggregation kernel.
//
// For each plan shape (the columns read and their types, the predicate's
// term shapes, the join key, the group keys, the aggregate inputs and
// classes, the cache size) this file writes a few dozen lines of CUDA that
// fix those choices at compile time, compiles them together with
// k_jit_lib.cuh / k_jit_kernel.cuh for sm_103a with NVRTC, loads the cubin
// with the runtime's library API and caches the kernel by its source text.
// Values that change between executions of one plan shape (column
// pointers, predicate bounds, tables, the dense key range) stay in the
// launch description, so re-running a plan reuses the compiled kernel.
//
// Host code only (no kernels of its own); the headers NVRTC needs are
// embedded at build time (vg_jit_headers.inc, written by build.py).
//
// The generated hooks restate, per plan: the predicate's comparisons after
// type promotion and its Kleene logic (vec_cmp / vec_bool_binary,
// src/scalar_ops.c:70-203), projected arithmetic (vec_arith,
// src/scalar_ops.c:11-66) and each accumulator's update (agg_accum_feed,
// src/agg_ops.c:93-158).

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include <nvrtc.h>

#include "k_groupby_dev.cuh"
#include "vg_jit_headers.inc"   // kJitHeaderNames[], kJitHeaderSources[], kJitHeaderCount

namespace {

// Launch shape: rows per thread, threads per CTA, CTAs per SM the register
// budget is set for, and whether the next rows' loads are issued before the
// current rows are processed.  VGPU_JIT_SHAPE="rows,threads,ctas[,pipe]"
// overrides it (tuning runs), and is compiled as given even if registers
// spill.
struct Shape { int rows = 2, threads = 1024, ctas = 1, pipe = 1; };

const Shape &shape() {
    static Shape sh;
    static bool init = false;
    if (!init) {
        const char *e = getenv("VGPU_JIT_SHAPE");
        int r, t, c, p = 1;
        if (e && sscanf(e, "%d,%d,%d,%d", &r, &t, &c, &p) >= 3 && (r == 2 || r == 4) && t >= 64 && t <= 1024 &&
            (t & 31) == 0 && c >= 1 && c <= 8 && (p == 0 || p == 1))
            sh.rows = r, sh.threads = t, sh.ctas = c, sh.pipe = p;
        init = true;
    }
    return sh;
}

// The shape a plan is compiled for: partition mode keeps four rows per
// thread in flight (each row's record position is a global atomic whose
// latency the other rows' hide).
// A dense group key read from a direct join's payload copy (the join +
// aggregate of a fact table against a dimension) runs two CTAs of 768
// threads per SM: 48 warps instead of 32 hide more of the payload reads'
// latency (measured on the 100M x 10M join + aggregate: 0.85 ms against
// 0.95 ms at 1024 x 1, when the 40-register budget still spilled a few
// words; with the rare rows deferred to the replay kernel it spills none).
bool occupancy_shape(const VgAggLaunch &L) {
    return !getenv("VGPU_JIT_SHAPE") && L.has_join && L.jpay && L.dense && L.jt.direct && !L.part && !L.sel;
}

Shape plan_shape(const VgAggLaunch &L) {
    Shape sh = shape();
    if (L.part && !getenv("VGPU_JIT_SHAPE")) sh.rows = 4;
    if (occupancy_shape(L)) {
        sh.rows = 2;
        sh.threads = 768;
        sh.ctas = 2;
        sh.pipe = 0;
    }
    return sh;
}

char g_jit_err[2048];

struct JitKernel {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kernel = nullptr;
    cudaKernel_t replay = nullptr;   // vg_jit_replay, in modules that defer rows
    int smem_set = 0;
    Shape shape;             // the launch shape it was compiled for
};

std::mutex g_mu;
std::unordered_map<std::string, JitKernel> g_cache;
unsigned long long g_compiles = 0;

void fmt(std::string &s, const char *f, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, f);
    vsnprintf(buf, sizeof(buf), f, ap);
    va_end(ap);
    s += buf;
}

std::string operand(const VgOperand &o) {
    std::string s;
    switch (o.side) {
    case VG_SIDE_PROBE:
        fmt(s, "InVal{X.p[%d][j], ((X.pok[%d] >> j) & 1u) != 0}", o.col, o.col);
        break;
    case VG_SIDE_BUILD:
        fmt(s, "InVal{X.b[%d][j], ((X.bok[%d] >> j) & 1u) != 0}", o.col, o.col);
        break;
    case VG_SIDE_LIT:
        fmt(s, "InVal{0x%llxull, true}", (unsigned long long)o.lit);
        break;
    default:
        s = "InVal{0ull, false}";
    }
    return s;
}

std::string value(const VgValue &v) {
    if (v.op == 0) return operand(v.a);
    std::string s;
    fmt(s, "vgj::arith<%d, %d, %d, %d>(%s, %s)", v.op, v.type, v.a.type, v.b.type, operand(v.a).c_str(),
        operand(v.b).c_str());
    return s;
}

int next_pow2(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

// Distinct aggregate input values of a plan (the values a partition record
// carries): acc_val[a] = index of accumulator a's input, -1 for n().
int record_values(const VgAggLaunch &L, int *acc_val, const VgValue **vals) {
    int nv = 0;
    for (int a = 0; a < L.n_accs; a++) {
        acc_val[a] = -1;
        if (L.acc[a].cls == VG_ACC_COUNT_ALL) continue;
        for (int v = 0; v < nv; v++)
            if (memcmp(vals[v], &L.acc[a].in, sizeof(VgValue)) == 0) acc_val[a] = v;
        if (acc_val[a] < 0) {
            vals[nv] = &L.acc[a].in;
            acc_val[a] = nv++;
        }
    }
    return nv;
}

}  // namespace

extern "C" {

const char *vgk_jit_error(void) { return g_jit_err; }
unsigned long long vgk_jit_compiles(void) { return g_compiles; }

// Shapes the specialised kernel covers: no replay, single-key joins with
// unique build keys (slot table), a shared-memory cache.
int vgk_agg_jit_ok(const VgAggLaunch *L) {
    if (getenv("VGPU_NO_JIT")) return 0;
    if (L->part) {
        if (L->replay || L->dense || L->n_keys != 1 || L->track_first) return 0;
    } else if (L->replay || L->cache_slots <= 0) {
        return 0;
    }
    if (L->has_join && (L->n_jkeys != 1 || !L->jt.slots || L->jt.rows)) return 0;
    if (L->has_join && L->join_kind != JOIN_INNER && L->join_kind != JOIN_LEFT) return 0;
    if (L->dense && (L->n_keys != 1 || L->dense_n + 1 > L->cache_slots)) return 0;
    return 1;
}

// Cache slots the specialised kernel uses: the dense range (rounded up to a
// power of two) when the keys are known, else up to twice the plan's cache
// size while the layout fits the shared memory one CTA per SM can have
// (the spill area holds two plan-size caches per SM).
int vgk_agg_jit_slots(const VgAggLaunch *L) {
    if (L->part) return 32;                // the NA-key group, one slot per warp
    if (L->dense) {
        int s = next_pow2(L->dense_n + 1);
        return s < 256 ? 256 : (s > L->cache_slots ? L->cache_slots : s);
    }
    int S = L->cache_slots;
    VgAggLaunch T = *L;
    for (;;) {
        const int S2 = 2 * S;
        if (S2 > 2 * L->cache_slots) break;
        T.cache_slots = S2;
        Lay c;
        make_lay(T, (uint64_t)S2, c);
        if (c.total > 200 * 1024) break;
        S = S2;
    }
    return S;
}

// The plan-specific source for L with S cache slots.
int vgk_agg_jit_source(const VgAggLaunch *L, int S, char *out, size_t out_bytes);

}  // extern "C"

namespace {

// A dense cache (it never misses) defers its rows for the global table.
bool defer_ok(const VgAggLaunch &L) { return L.dense && !L.part && L.defer_bits && L.defer_n; }

std::string gen_source(const VgAggLaunch &L, int S, bool vec, const Shape &sh) {
    VgAggLaunch T = L;
    T.cache_slots = S;
    Lay c;
    make_lay(T, (uint64_t)S, c);
    std::string s;
    s += "// generated by jit_agg.cu\n";
    fmt(s, "#define VGJ_R %d\n#define VGJ_NPC %d\n#define VGJ_NBC %d\n", sh.rows, L.n_pcols,
        L.has_join ? L.n_bcols : 0);
    s += "#include \"k_jit_lib.cuh\"\n";
    fmt(s, "#define VGJ_THREADS %d\n#define VGJ_MINB %d\n#define VGJ_S %d\n", sh.threads, sh.ctas, S);
    fmt(s, "#define VGJ_SEL %d\n#define VGJ_VEC %d\n#define VGJ_PIPE %d\n", L.sel ? 1 : 0, vec ? 1 : 0,
        (!L.sel && sh.pipe) ? 1 : 0);
    fmt(s, "#define VGJ_PRED %d\n#define VGJ_JOIN %d\n#define VGJ_PAY %d\n", L.pred.n_terms > 0 ? 1 : 0,
        L.has_join ? 1 : 0, (L.has_join && L.jpay && L.jpay_n == L.n_bcols && L.n_bcols >= 1) ? 1 : 0);
    if (L.has_join)
        fmt(s, "#define VGJ_JKIND %d\n#define VGJ_JCOL %d\n#define VGJ_JCONV %d\n#define VGJ_JKT %d\n"
               "#define VGJ_JDIRECT %d\n",
            L.join_kind, L.jkey_col[0], L.jkey_conv[0], L.jt.key_types[0], L.jt.direct ? 1 : 0);
    // compact payload entries (VgJPay16): which column is narrowed, and its type
    {
        const int p16 = (L.has_join && L.jpay && L.jpay16 && L.jt.direct) ? 1 : 0;
        const int nar = p16 ? L.jpay_narrow : -1;
        fmt(s, "#define VGJ_PAY16 %d\n#define VGJ_PAY_NARROW %d\n#define VGJ_PAY_NARROW_T %d\n", p16, nar,
            nar >= 0 ? L.bcols[nar].type : 0);
    }
    fmt(s, "#define VGJ_NK %d\n#define VGJ_DENSE %d\n#define VGJ_TRACK %d\n#define VGJ_PART %d\n", L.n_keys,
        L.dense ? 1 : 0, L.track_first ? 1 : 0, L.part ? 1 : 0);
    // a dense cache with an n() accumulator: a slot is live when its count
    // is nonzero (no per-row state store)
    {
        int live_acc = -1;
        if (L.dense && !L.part)
            for (int a = 0; a < L.n_accs && live_acc < 0; a++)
                if (L.acc[a].cls == VG_ACC_COUNT_ALL) live_acc = a;
        fmt(s, "#define VGJ_LIVE_BY_CNT %d\n#define VGJ_LIVE_CNT %lluu\n", live_acc >= 0 ? 1 : 0,
            live_acc >= 0 ? (unsigned long long)c.cnt[live_acc] : 0ull);
    }
    // a dense cache's rows for the global table, deferred to the replay kernel
    {
        uint32_t f64 = 0;
        for (int a = 0; a < L.n_accs; a++)
            if (L.acc[a].cls == VG_ACC_SUM_F64) f64 |= 1u << a;
        fmt(s, "#define VGJ_DEFER %d\n#define VGJ_F64_MASK %uu\n", defer_ok(L) ? 1 : 0, f64);
    }
    // rows that pass a filter queued per warp (few of a step's rows pass)
    fmt(s, "#define VGJ_COMPACT %d\n",
        (L.pred.n_terms > 0 && !L.has_join && !L.part && !L.sel && !L.track_first && !L.dense) ? 1 : 0);
    // per-CTA record ranges; holes when a filter or an inner join drops rows
    fmt(s, "#define VGJ_PART_CTA %d\n#define VGJ_PART_HOLES %d\n#define VGJ_OFF_PCUR %lluu\n",
        (L.part && L.po.cta_off) ? 1 : 0,
        (L.pred.n_terms > 0 || (L.has_join && L.join_kind == JOIN_INNER)) ? 1 : 0, (unsigned long long)c.total);
    fmt(s, "#define VGJ_OFF_STATE %lluu\n#define VGJ_OFF_NM %lluu\n#define VGJ_OFF_KEYS %lluu\n"
           "#define VGJ_OFF_FIRST %lluu\n",
        (unsigned long long)c.state, (unsigned long long)c.nm, (unsigned long long)c.keys,
        (unsigned long long)c.first);
    s += "using namespace vgj;\n";

    // probe columns
    s += "VG_DEV void vgj_load_probe(const VgAggLaunch &L, Rows &X, int64_t r0, int nv, bool vec, "
         "const int64_t (&phys)[R], uint32_t want) {\n";
    for (int i = 0; i < L.n_pcols; i++) {
        if (L.sel)
            fmt(s, "    load_rows<%d>(L.pcols[%d], phys, want, X.p[%d], X.pok[%d]);\n", L.pcols[i].type, i, i, i);
        else
            fmt(s, "    load_dense<%d>(L.pcols[%d], r0, nv, vec, X.p[%d], X.pok[%d]);\n", L.pcols[i].type, i, i, i);
    }
    s += "    (void)L; (void)X; (void)r0; (void)nv; (void)vec; (void)phys; (void)want;\n}\n";

    // predicate
    s += "VG_DEV uint32_t vgj_pred(const VgAggLaunch &L, const Rows &X) {\n    uint32_t m = 0xFFFFFFFFu;\n";
    for (int t = 0; t < L.pred.n_terms; t++) {
        const VgTerm &tm = L.pred.term[t];
        fmt(s, "    m &= term_mask<%d, %d, %d, %d, %d>(L, X);\n", tm.kind, tm.kind == VG_TERM_NONE ? 0 : tm.col,
            tm.domain, tm.nan_keep ? 1 : 0, t);
    }
    s += "    (void)L; (void)X;\n    return m;\n}\n";

    // build columns
    s += "VG_DEV void vgj_load_build(const VgAggLaunch &L, Rows &X, const int64_t (&brow)[R], uint32_t want) {\n";
    if (L.has_join)
        for (int i = 0; i < L.n_bcols; i++)
            fmt(s, "    load_rows<%d>(L.bcols[%d], brow, want, X.b[%d], X.bok[%d]);\n", L.bcols[i].type, i, i, i);
    s += "    (void)L; (void)X; (void)brow; (void)want;\n}\n";

    // group keys
    s += "VG_DEV void vgj_keys(const Rows &X, int j, Keys &k, uint32_t &nm) {\n";
    for (int i = 0; i < L.n_keys; i++)
        fmt(s, "    { InVal v = %s; if (v.ok) k.w[%d] = vg_norm_key(v.bits, %d); else nm |= %uu; }\n",
            value(L.key[i]).c_str(), i, L.key[i].type, 1u << i);
    s += "    (void)X; (void)j; (void)k; (void)nm;\n}\n";

    // cache updates
    s += "VG_DEV uint32_t vgj_cache_update(char *sm, int slot, const Rows &X, int j, VgjBases &wb) {\n"
         "    uint32_t fail = 0;\n";
    for (int a = 0; a < L.n_accs; a++) {
        const VgAccSpec &A = L.acc[a];
        const int count = (L.skip_count_mask >> a) & 1u ? 0 : 1;
        std::string v = A.cls == VG_ACC_COUNT_ALL ? std::string("InVal{0ull, true}") : value(A.in);
        fmt(s, "    if (!cache_acc_k<%d, %d, %d, %d, %lluu, %lluu, %lluu, %lluu, %lluu, %d>(sm, slot, %s, wb)) "
               "fail |= %uu;\n",
            a, A.cls, A.na_rm ? 1 : 0, count, (unsigned long long)c.cnt[a], (unsigned long long)c.val[a],
            (unsigned long long)c.flags[a], (unsigned long long)c.base[a], (unsigned long long)c.win[a], S,
            v.c_str(), 1u << a);
    }
    s += "    (void)sm; (void)slot; (void)X; (void)j; (void)wb;\n    return fail;\n}\n";

    // the CTA's window bases into a live slot's base words (kernel tail)
    s += "VG_DEV void vgj_fix_bases(char *sm, int slot) {\n";
    for (int a = 0; a < L.n_accs; a++)
        if (L.acc[a].cls == VG_ACC_SUM_F64)
            fmt(s, "    ((int32_t *)(sm + %lluu))[slot] = vgj_cta_base[%d];\n", (unsigned long long)c.base[a], a);
    s += "    (void)sm; (void)slot;\n}\n";

    // global-table updates of the accumulators in `which`
    s += "VG_DEV void vgj_global_update(const VgAggLaunch &L, int64_t g, const Rows &X, int j, uint32_t which) {\n";
    for (int a = 0; a < L.n_accs; a++) {
        const VgAccSpec &A = L.acc[a];
        std::string v = A.cls == VG_ACC_COUNT_ALL ? std::string("InVal{0ull, true}") : value(A.in);
        fmt(s, "    if (which & %uu) acc_update<true>(L.acc[%d], global_ptrs(L.gt, %d), L.gt.cap, g, %s);\n", 1u << a,
            a, a, v.c_str());
    }
    s += "    (void)L; (void)g; (void)X; (void)j; (void)which;\n}\n";

    // spill of single accumulators (global table full)
    s += "VG_DEV void vgj_spill(const VgAggLaunch &L, int64_t li, uint32_t which) {\n";
    for (int a = 0; a < L.n_accs; a++) fmt(s, "    if (which & %uu) spill_row(L, li, 0, %d);\n", 1u << a, a);
    s += "    (void)L; (void)li; (void)which;\n}\n";

    // partition mode: a row with a valid key becomes a record in its bucket
    // (cursors padded to one per 128-byte line: VG_PAGG_CURSOR_STRIDE)
    s += "VG_DEV unsigned long long vgj_reserve(const VgAggLaunch &L, char *sm, uint64_t key) {\n";
    if (L.part) {
        s += "    const uint64_t ow = key ^ 0x8000000000000000ull;\n"
             "    const uint64_t d = ow < L.po.omin ? 0ull : ((ow - L.po.omin) >> L.po.shift);\n"
             "    const uint32_t b = d >= (uint64_t)L.po.n_buckets ? (uint32_t)(L.po.n_buckets - 1) : (uint32_t)d;\n";
        if (L.po.cta_off)
            s += "    const unsigned long long pos = atomicAdd((uint32_t *)(sm + VGJ_OFF_PCUR) + b, 1u);\n"
                 "    return pos < L.po.total ? pos : ~0ull;\n";
        else
            s += "    const unsigned long long pos = atomicAdd(L.po.cursor + (uint64_t)b * VG_PAGG_CURSOR_STRIDE, 1ull);\n"
                 "    (void)sm;\n    return pos < __ldg(L.po.end + b) ? pos : ~0ull;\n";
    } else {
        s += "    (void)L; (void)sm; (void)key;\n    return ~0ull;\n";
    }
    s += "}\n";
    s += "VG_DEV void vgj_write(const VgAggLaunch &L, unsigned long long pos, uint64_t key, const Rows &X, int j) {\n";
    if (L.part) {
        int acc_val[VG_MAX_ACCS];
        const VgValue *vals[VG_MAX_ACCS];
        const int nv = record_values(L, acc_val, vals);
        const int rw = 2 + nv + (nv & 1);
        s += "    if (pos == ~0ull) { atomicOr(L.po.err, VG_ERR_FULL); return; }\n";
        for (int v = 0; v < nv; v++) fmt(s, "    const InVal v%d = %s;\n", v, value(*vals[v]).c_str());
        s += "    uint64_t fl = 0;\n";
        for (int v = 0; v < nv; v++) fmt(s, "    if (v%d.ok) fl |= %lluull;\n", v, 1ull << v);
        // the record's words: 32-byte stores when records are a multiple of
        // 4 words (so every record starts 32-byte aligned), else 16-byte ones
        std::vector<std::string> w;
        w.push_back("key");
        w.push_back("fl");
        for (int v = 0; v < nv; v++) w.push_back("v" + std::to_string(v) + ".bits");
        while ((int)w.size() < rw) w.push_back("0ull");
        fmt(s, "    uint64_t *r = L.po.rec + pos * %dull;\n", rw);
        int i = 0;
        if (rw % 4 == 0)
            for (; i + 4 <= rw; i += 4)
                fmt(s, "    vg_st256(r + %d, %s, %s, %s, %s);\n", i, w[i].c_str(), w[i + 1].c_str(), w[i + 2].c_str(),
                    w[i + 3].c_str());
        for (; i < rw; i += 2)
            fmt(s, "    *(ulonglong2 *)(r + %d) = make_ulonglong2(%s, %s);\n", i, w[i].c_str(), w[i + 1].c_str());
    }
    s += "    (void)L; (void)pos; (void)key; (void)X; (void)j;\n}\n";

    s += "#include \"k_jit_kernel.cuh\"\n";
    return s;
}

// NVRTC: source -> cubin.  *spill: bytes of register spill stores ptxas
// reported; *log_out (optional): the compile log.
int nvrtc_cubin(const std::string &src, std::vector<char> &cubin, int *spill, std::string *log_out) {
    nvrtcProgram prog;
    nvrtcResult r = nvrtcCreateProgram(&prog, src.c_str(), "vg_jit_agg.cu", kJitHeaderCount, kJitHeaderSources,
                                       kJitHeaderNames);
    if (r != NVRTC_SUCCESS) {
        snprintf(g_jit_err, sizeof(g_jit_err), "nvrtcCreateProgram: %s", nvrtcGetErrorString(r));
        return -1;
    }
    const char *opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "--generate-line-info", "--ptxas-options=-v"};
    r = nvrtcCompileProgram(prog, 4, opts);
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    std::vector<char> log(n + 1, 0);
    nvrtcGetProgramLog(prog, log.data());
    if (log_out) *log_out = log.data();
    if (r != NVRTC_SUCCESS) {
        snprintf(g_jit_err, sizeof(g_jit_err), "NVRTC: %s\n%.1800s", nvrtcGetErrorString(r), log.data());
        nvrtcDestroyProgram(&prog);
        return -1;
    }
    const char *sp = strstr(log.data(), "bytes spill stores");
    int spills = 0;
    if (sp) {
        const char *q = sp;
        while (q > log.data() && q[-1] == ' ') q--;
        while (q > log.data() && q[-1] >= '0' && q[-1] <= '9') q--;
        spills = atoi(q);
    }
    *spill = spills;
    nvrtcGetCUBINSize(prog, &n);
    cubin.resize(n);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    g_compiles++;
    return 0;
}

// Compiles the plan at the preferred launch shape; if ptxas had to spill
// registers there, at half the threads per CTA (twice the registers per
// thread), down to 256.  out.shape records the shape compiled for.
int compile_plan(const VgAggLaunch &L, int S, bool vec, std::vector<char> &cubin, Shape &used,
                 std::string *log_out) {
    Shape sh = plan_shape(L);
    std::string src;
    for (;;) {
        int spill = 0;
        src = gen_source(L, S, vec, sh);
        if (nvrtc_cubin(src, cubin, &spill, log_out) != 0) return -1;
        if (spill == 0 || sh.threads <= 256 || getenv("VGPU_JIT_SHAPE")) break;   // an explicit shape is kept
        if (sh.ctas == 2 && sh.threads == 768) {
            // the two-CTA shape: a few spilled words are fine, more fall
            // back to one CTA of 1024 threads
            if (spill <= 64) break;
            sh = Shape();
            continue;
        }
        sh.threads /= 2;
    }
    // VGPU_JIT_DUMP=<file>: append the source of each plan compiled
    if (const char *dump = getenv("VGPU_JIT_DUMP")) {
        if (FILE *f = fopen(dump, "a")) {
            fputs(src.c_str(), f);
            fclose(f);
        }
    }
    used = sh;
    return 0;
}

int load_kernel(const std::vector<char> &cubin, JitKernel &out, const char *name = "vg_jit_agg") {
    cudaError_t e = cudaLibraryLoadData(&out.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) {
        snprintf(g_jit_err, sizeof(g_jit_err), "cudaLibraryLoadData: %s", cudaGetErrorString(e));
        return -1;
    }
    e = cudaLibraryGetKernel(&out.kernel, out.lib, name);
    if (e != cudaSuccess) {
        snprintf(g_jit_err, sizeof(g_jit_err), "cudaLibraryGetKernel: %s", cudaGetErrorString(e));
        return -1;
    }
    return 0;
}

// Grid and rows per tile of a launch over n rows (CTA c processes tiles c,
// c + grid, ...): at most two CTAs per SM (the spill area holds two caches
// per SM).
void launch_geometry(const Shape &sh, int64_t n, int *grid, int64_t *tile) {
    const int sms = vgk_num_sms();
    const int64_t per = (int64_t)sh.rows * sh.threads;
    const int64_t tiles = (n + per - 1) / per;
    const int64_t cap = (int64_t)sms * (sh.ctas < 2 ? sh.ctas : 2);
    *grid = (int)(tiles < cap ? (tiles < 1 ? 1 : tiles) : cap);
    *tile = per;
}

bool vec_ok(const VgAggLaunch &L) {
    if (L.sel) return false;
    for (int c = 0; c < L.n_pcols; c++) {
        const uintptr_t p = (uintptr_t)L.pcols[c].data;
        if (L.pcols[c].type == VEC_BOOL ? (p & 3) : (p & 15)) return false;
    }
    return true;
}

}  // namespace

extern "C" {

int vgk_agg_jit_source(const VgAggLaunch *L, int S, char *out, size_t out_bytes) {
    std::string s = gen_source(*L, S, vec_ok(*L), plan_shape(*L));
    if (s.size() + 1 > out_bytes) return (int)(s.size() + 1);
    memcpy(out, s.c_str(), s.size() + 1);
    return 0;
}

// Compiles the kernel for L without launching it (no device needed):
// 0 on success, -1 with vgk_jit_error() set.
int vgk_agg_jit_compile_only(const VgAggLaunch *L, int *regs_out) {
    const int S = vgk_agg_jit_slots(L);
    std::vector<char> cubin;
    Shape used;
    std::string log;
    const int rc = compile_plan(*L, S, vec_ok(*L), cubin, used, &log);
    snprintf(g_jit_err, sizeof(g_jit_err), "%sthreads per CTA: %d\n%.1800s", rc == 0 ? "" : "NVRTC failed:\n",
             used.threads, log.c_str());
    if (regs_out) {
        const char *p = strstr(log.c_str(), "Used ");
        *regs_out = p ? atoi(p + 5) : -1;
    }
    return rc;
}

// Launches the specialised kernel over n_logical rows: 1 launched, 0 the
// plan shape is not covered (nothing launched), -1 error (message in
// vgk_jit_error()).
}  // extern "C"

namespace {

// The compiled kernel of plan L (cached by its source), or null
// (vgk_jit_error()).
// The code-generation signature of a launch: the launch with every
// pointer reduced to whether it is set and the per-batch numbers that the
// kernel reads at run time (row counts and bases, capacities, the direct
// table's minimum, partition bounds) cleared, plus S, vec and the shape.
// gen_source reads pointers only to test them for NULL and those numbers
// only as kernel parameters, so launches with one signature share one
// source; the source (tens of kilobytes of text) is then generated and
// looked up once per signature instead of once per launch.
template <typename T> void set_flag(T *&p) { p = p ? (T *)(uintptr_t)1 : nullptr; }
template <typename T> void shift_ptr(T *&p, uintptr_t d) { if (p) p = (T *)((uintptr_t)p + d); }

std::string launch_signature(const VgAggLaunch &L, int S, bool vec, const Shape &sh) {
    VgAggLaunch T;
    memcpy(&T, &L, sizeof(T));
    T.n_rows = T.sel_n = T.row_base = 0;
    set_flag(T.sel);
    for (int i = 0; i < VG_MAX_COLS; i++) {
        set_flag(T.pcols[i].data);
        set_flag(T.pcols[i].valid);
        set_flag(T.bcols[i].data);
        set_flag(T.bcols[i].valid);
    }
    T.jt.cap = 0;
    T.jt.dmin = 0;
    T.jt.n_build = 0;
    set_flag(T.jt.slots);
    set_flag(T.jt.state);
    set_flag(T.jt.keys);
    set_flag(T.jt.start);
    set_flag(T.jt.count);
    set_flag(T.jt.rows);
    set_flag(T.jt.err);
    T.gt.cap = 0;
    set_flag(T.gt.state);
    set_flag(T.gt.nullmask);
    set_flag(T.gt.keys);
    set_flag(T.gt.first_row);
    for (int a = 0; a < VG_MAX_ACCS; a++) {
        set_flag(T.gt.cnt[a]);
        set_flag(T.gt.val[a]);
        set_flag(T.gt.flags[a]);
        set_flag(T.gt.lacc[a]);
    }
    set_flag(T.gt.n_used);
    set_flag(T.gt.err);
    set_flag(T.spill_rows);
    set_flag(T.spill_rows_n);
    set_flag(T.spill_cache);
    set_flag(T.spill_cache_n);
    set_flag(T.replay);
    T.spill_rows_cap = T.spill_cache_cap = T.replay_n = T.batch_idx = T.li_base = 0;
    T.dense_min = 0;
    set_flag(T.jpay);
    T.jpay_min = 0;
    set_flag(T.po.rec);
    set_flag(T.po.cursor);
    set_flag(T.po.end);
    set_flag(T.po.err);
    set_flag(T.po.cta_off);
    set_flag(T.po.start);
    T.po.omin = 0;
    T.po.shift = 0;
    T.po.n_buckets = 0;
    T.po.total = 0;
    set_flag(T.defer_bits);
    set_flag(T.defer_n);
    T.defer_words = 0;
    std::string sig((const char *)&T, sizeof(T));
    const int extra[6] = {S, vec ? 1 : 0, sh.rows, sh.threads, sh.ctas, sh.pipe};
    sig.append((const char *)extra, sizeof(extra));
    return sig;
}

std::unordered_map<std::string, JitKernel *> g_by_sig;

JitKernel *plan_kernel(const VgAggLaunch *L, int S, bool vec) {
    const Shape sh = plan_shape(*L);
    const std::string sig = launch_signature(*L, S, vec, sh);
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto hit = g_by_sig.find(sig);
        if (hit != g_by_sig.end()) return hit->second;
    }
    std::string src = gen_source(*L, S, vec, sh);
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_cache.find(src);
    if (it == g_cache.end()) {
        JitKernel k;
        std::vector<char> cubin;
        if (compile_plan(*L, S, vec, cubin, k.shape, nullptr) != 0) return nullptr;
        if (load_kernel(cubin, k) != 0) return nullptr;
        if (defer_ok(*L)) {
            cudaError_t e = cudaLibraryGetKernel(&k.replay, k.lib, "vg_jit_replay");
            if (e != cudaSuccess) {
                snprintf(g_jit_err, sizeof(g_jit_err), "cudaLibraryGetKernel(vg_jit_replay): %s",
                         cudaGetErrorString(e));
                return nullptr;
            }
        }
        it = g_cache.emplace(src, k).first;
    }
    g_by_sig.emplace(sig, &it->second);     // elements of g_cache never move
    return &it->second;
}

}  // namespace

extern "C" {

int vgk_agg_jit_geometry(const VgAggLaunch *L, int64_t n, int *grid, int64_t *tile) {
    if (!vgk_agg_jit_ok(L)) {
        snprintf(g_jit_err, sizeof(g_jit_err), "plan not covered by the specialised kernel");
        return -1;
    }
    JitKernel *jk = plan_kernel(L, vgk_agg_jit_slots(L), vec_ok(*L));
    if (!jk) return -1;
    launch_geometry(jk->shape, n, grid, tile);
    return 0;
}

int vgk_agg_launch_jit(const VgAggLaunch *L, int64_t n_logical, vg_stream_t s) {
    if (!vgk_agg_jit_ok(L)) return 0;
    const int S = vgk_agg_jit_slots(L);
    const bool vec = vec_ok(*L);
    JitKernel *jk = plan_kernel(L, S, vec);
    if (!jk) return -1;
    VgAggLaunch T = *L;
    T.cache_slots = S;
    Lay c;
    make_lay(T, (uint64_t)S, c);
    int smem = (int)c.total;
    if (L->part && L->po.cta_off) smem += 4 * L->po.n_buckets;      // per-CTA bucket counters
    if (jk->smem_set < smem) {
        cudaError_t e = cudaFuncSetAttribute((const void *)jk->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             smem);
        if (e != cudaSuccess) {
            snprintf(g_jit_err, sizeof(g_jit_err), "jit smem attribute: %s", cudaGetErrorString(e));
            return -1;
        }
        jk->smem_set = smem;
    }
    int grid = 0;
    int64_t per = 0;
    launch_geometry(jk->shape, n_logical, &grid, &per);
    const Shape &sh = jk->shape;
    cudaStream_t st = (cudaStream_t)s;
    int64_t n = n_logical;
    void *args[] = {(void *)&T, (void *)&n};
    vg_prof_begin(VG_PROF_AGG, st);
    cudaError_t e = cudaLaunchKernel((const void *)jk->kernel, dim3(grid), dim3(sh.threads), args, (size_t)smem, st);
    vg_launch_counter++;
    // the rows this launch deferred (a dense cache): applied right after it
    if (e == cudaSuccess && jk->replay) {
        e = cudaLaunchKernel((const void *)jk->replay, dim3(2 * vgk_num_sms()), dim3(256), args, 0, st);
        vg_launch_counter++;
    }
    vg_prof_end(VG_PROF_AGG, st);
    if (e != cudaSuccess) {
        snprintf(g_jit_err, sizeof(g_jit_err), "jit agg launch: %s", cudaGetErrorString(e));
        return -1;
    }
    return 1;
}

}  // extern "C"

// ---------------------------------------------------------------------
// partitioned aggregation, second step: the bucket reducer (k_jit_pagg.cuh)
// ---------------------------------------------------------------------
namespace {

// Shared-memory layout of the reducer for G groups and S hash slots:
// only the arrays an accumulator class touches are allocated.
struct PLay {
    uint64_t hid, gkey, total;
    uint64_t cnt[VG_MAX_ACCS], val[VG_MAX_ACCS], flags[VG_MAX_ACCS], base[VG_MAX_ACCS], win[VG_MAX_ACCS];
};

bool acc_counted(const VgAggLaunch &L, int a) {
    const int cls = L.acc[a].cls;
    if (cls == VG_ACC_COUNT_ALL || cls == VG_ACC_COUNT_VALID) return true;
    if (cls == VG_ACC_SUM_I64 || cls == VG_ACC_SUM_F64) return !((L.skip_count_mask >> a) & 1u);
    return false;
}

PLay pagg_lay(const VgAggLaunch &L, int G, int S) {
    PLay c;
    memset(&c, 0, sizeof(c));
    uint64_t off = 0;
    auto take = [&](uint64_t bytes) {
        const uint64_t o = off;
        off = (off + bytes + 15) & ~15ull;
        return o;
    };
    c.hid = take(4ull * S);
    c.gkey = take(8ull * G);
    for (int a = 0; a < L.n_accs; a++) {
        const int cls = L.acc[a].cls;
        if (acc_counted(L, a)) c.cnt[a] = take(4ull * G);
        if (cls == VG_ACC_SUM_I64 || acc_is_min(cls) || acc_is_max(cls)) c.val[a] = take(8ull * G);
        if (cls != VG_ACC_COUNT_ALL && cls != VG_ACC_COUNT_VALID) c.flags[a] = take(4ull * G);
        if (cls == VG_ACC_SUM_F64) {
            c.base[a] = take(4ull * G);
            c.win[a] = take(8ull * G * kWin);
        }
    }
    c.total = off;
    return c;
}

constexpr uint64_t kPaggSmem = 226 * 1024;   // dynamic shared memory of one reducer CTA

int hash_slots(int G) { return next_pow2(2 * G); }

std::string gen_pagg_source(const VgAggLaunch &L, const VgFinish *fin, int n_out, int G, int threads,
                            int minb = 1) {
    const int S = hash_slots(G);
    const PLay c = pagg_lay(L, G, S);
    int acc_val[VG_MAX_ACCS];
    const VgValue *vals[VG_MAX_ACCS];
    const int nv = record_values(L, acc_val, vals);
    const int rw = 2 + nv + (nv & 1);
    std::string s;
    s += "// generated by jit_agg.cu (partitioned aggregation, bucket reducer)\n";
    s += "#define VGJ_R 2\n#define VGJ_NPC 1\n#define VGJ_NBC 1\n#include \"k_jit_lib.cuh\"\n";
    fmt(s, "#define VGP_G %d\n#define VGP_S %d\n#define VGP_RW %d\n#define VGP_THREADS %d\n#define VGP_MINB %d\n", G,
        S, rw, threads, minb);
    fmt(s, "#define VGP_OFF_HID %lluu\n#define VGP_OFF_GKEY %lluu\n", (unsigned long long)c.hid,
        (unsigned long long)c.gkey);
    s += "#include \"k_jit_pagg.cuh\"\n";

    // initial accumulator state of a new group
    s += "VG_DEV void vgp_init(char *sm, int g) {\n";
    for (int a = 0; a < L.n_accs; a++) {
        const int cls = L.acc[a].cls;
        if (acc_counted(L, a)) fmt(s, "    ((uint32_t *)(sm + %lluu))[g] = 0u;\n", (unsigned long long)c.cnt[a]);
        if (cls != VG_ACC_COUNT_ALL && cls != VG_ACC_COUNT_VALID)
            fmt(s, "    ((uint32_t *)(sm + %lluu))[g] = 0u;\n", (unsigned long long)c.flags[a]);
        if (cls == VG_ACC_SUM_I64)
            fmt(s, "    ((uint32_t *)(sm + %lluu))[g] = 0u; ((int32_t *)(sm + %lluu))[g] = 0;\n",
                (unsigned long long)c.val[a], (unsigned long long)(c.val[a] + 4ull * G));
        else if (acc_is_min(cls))
            fmt(s, "    ((int64_t *)(sm + %lluu))[g] = 0x7FFFFFFFFFFFFFFFll;\n", (unsigned long long)c.val[a]);
        else if (acc_is_max(cls))
            fmt(s, "    ((int64_t *)(sm + %lluu))[g] = (int64_t)0x8000000000000000ull;\n",
                (unsigned long long)c.val[a]);
        if (cls == VG_ACC_SUM_F64) {
            fmt(s, "    ((int32_t *)(sm + %lluu))[g] = kBaseUnset;\n", (unsigned long long)c.base[a]);
            fmt(s, "    for (int i = 0; i < 2 * kWin; i++) ((uint32_t *)(sm + %lluu))[i * %d + g] = 0u;\n",
                (unsigned long long)c.win[a], G);
        }
    }
    s += "    (void)sm; (void)g;\n}\n";

    // one record into its group
    s += "VG_DEV void vgp_acc(char *sm, int g, const uint64_t (&w)[VGP_RW], const VgPaggReduce &B, uint64_t fpos) {\n";
    s += "    const uint64_t fl = w[1];\n";
    for (int a = 0; a < L.n_accs; a++) {
        const VgAccSpec &A = L.acc[a];
        std::string x = acc_val[a] < 0 ? std::string("InVal{0ull, true}")
                                       : std::string("InVal{w[") + std::to_string(2 + acc_val[a]) + "], ((fl >> " +
                                             std::to_string(acc_val[a]) + ") & 1ull) != 0}";
        const int count = acc_counted(L, a) ? 1 : 0;
        fmt(s, "    { const InVal x = %s;\n", x.c_str());
        fmt(s, "      if (!vgj::cache_acc<%d, %d, %d, %lluu, %lluu, %lluu, %lluu, %lluu, %d>(sm, g, x)) {\n", A.cls,
            A.na_rm ? 1 : 0, count, (unsigned long long)c.cnt[a], (unsigned long long)c.val[a],
            (unsigned long long)c.flags[a], (unsigned long long)c.base[a], (unsigned long long)c.win[a], G);
        if (A.cls == VG_ACC_SUM_F64) {
            fmt(s, "          vgp::sum_fallback(B.fs[%d] + fpos, B.fc[%d] + fpos, (uint32_t *)(sm + %lluu) + g, "
                   "vg_bits_to_f64(x.bits), B.err);\n",
                a, a, (unsigned long long)c.flags[a]);
            if (count) fmt(s, "          atomicAdd((uint32_t *)(sm + %lluu) + g, 1u);\n", (unsigned long long)c.cnt[a]);
        }
        s += "      } }\n";
    }
    s += "    (void)sm; (void)g; (void)w; (void)B; (void)fpos; (void)fl;\n}\n";

    // outputs of a group
    s += "VG_DEV uint32_t vgp_finish(const char *sm, int g, const VgPaggReduce &B, uint64_t fpos, uint64_t opos) {\n";
    s += "    uint32_t okb = 0;\n";
    for (int o = 0; o < n_out; o++) {
        const VgFinish &F = fin[o];
        const int a = F.acc;
        const int cls = L.acc[a].cls;
        std::string fsp = cls == VG_ACC_SUM_F64 ? "B.fs[" + std::to_string(a) + "] + fpos" : std::string("nullptr");
        std::string fcp = cls == VG_ACC_SUM_F64 ? "B.fc[" + std::to_string(a) + "] + fpos" : std::string("nullptr");
        fmt(s, "    { bool ok; const double r = vgp::finish<%d, %d, %d, %lluu, %lluu, %lluu, %lluu, %lluu>(sm, g, %s, %s, "
               "ok, B.warn);\n",
            F.finish, cls, F.in_type, (unsigned long long)c.cnt[a], (unsigned long long)c.val[a],
            (unsigned long long)c.flags[a], (unsigned long long)c.base[a], (unsigned long long)c.win[a], fsp.c_str(),
            fcp.c_str());
        fmt(s, "      B.st_out[%d][opos] = ok ? r : 0.0; if (ok) okb |= %uu; }\n", o, 1u << o);
    }
    s += "    (void)sm; (void)g; (void)B; (void)fpos; (void)opos;\n    return okb;\n}\n";
    return s;
}

}  // namespace

extern "C" {

// Groups one reducer CTA holds for this plan (0: the plan does not fit).
int vgk_pagg_groups_for(const VgAggLaunch *L, int ctas) {
    // each CTA on an SM also holds about 1 KiB of the SM's shared memory
    const uint64_t limit = ctas <= 1 ? kPaggSmem : kPaggSmem / (uint64_t)ctas - 1024;
    for (int G = 4096; G >= 256; G -= 256) {
        const PLay c = pagg_lay(*L, G, hash_slots(G));
        if (c.total <= limit) return G;
    }
    return 0;
}

int vgk_pagg_groups(const VgAggLaunch *L) { return vgk_pagg_groups_for(L, 1); }

// Record words of the plan's partition records.
int vgk_pagg_record_words(const VgAggLaunch *L) {
    int acc_val[VG_MAX_ACCS];
    const VgValue *vals[VG_MAX_ACCS];
    const int nv = record_values(*L, acc_val, vals);
    return 2 + nv + (nv & 1);
}

int vgk_pagg_source(const VgAggLaunch *L, const VgFinish *fin, int n_out, int G, char *out, size_t out_bytes) {
    std::string s = gen_pagg_source(*L, fin, n_out, G, 1024);
    if (s.size() + 1 > out_bytes) return (int)(s.size() + 1);
    memcpy(out, s.c_str(), s.size() + 1);
    return 0;
}

// Compiles (cached) and launches the bucket reducer: one CTA per SM.
// 0 on success, -1 with vgk_jit_error() set.
int vgk_pagg_reduce(const VgAggLaunch *L, const VgFinish *fin, int n_out, int G, int ctas, const VgPaggReduce *B,
                    vg_stream_t s) {
    if (getenv("VGPU_NO_JIT")) {
        snprintf(g_jit_err, sizeof(g_jit_err), "partitioned aggregation needs the run-time compiler");
        return -1;
    }
    if (ctas != 2 && ctas != 4 && ctas != 8) ctas = 1;
    int threads = 1024 / ctas;
    std::string src = gen_pagg_source(*L, fin, n_out, G, threads, ctas);
    JitKernel *jk;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto it = g_cache.find(src);
        if (it == g_cache.end()) {
            JitKernel k;
            std::vector<char> cubin;
            int spill = 0;
            if (nvrtc_cubin(src, cubin, &spill, nullptr) != 0) return -1;
            if (spill > 256) {
                // fewer threads, more registers each
                threads /= 2;
                if (nvrtc_cubin(gen_pagg_source(*L, fin, n_out, G, threads, ctas), cubin, &spill, nullptr) != 0)
                    return -1;
            }
            k.shape.threads = threads;
            if (load_kernel(cubin, k, "vg_jit_pagg") != 0) return -1;
            it = g_cache.emplace(src, k).first;
        }
        jk = &it->second;
    }
    const int smem = (int)pagg_lay(*L, G, hash_slots(G)).total;
    if (jk->smem_set < smem) {
        cudaError_t e = cudaFuncSetAttribute((const void *)jk->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             smem);
        if (e != cudaSuccess) {
            snprintf(g_jit_err, sizeof(g_jit_err), "pagg smem attribute: %s", cudaGetErrorString(e));
            return -1;
        }
        jk->smem_set = smem;
    }
    const int cap = vgk_num_sms() * ctas;
    const int grid = B->n_buckets < cap ? (B->n_buckets < 1 ? 1 : B->n_buckets) : cap;
    cudaStream_t st = (cudaStream_t)s;
    VgPaggReduce T = *B;
    void *args[] = {(void *)&T};
    vg_prof_begin(VG_PROF_PAGG, st);
    cudaError_t e = cudaLaunchKernel((const void *)jk->kernel, dim3(grid), dim3(jk->shape.threads), args, (size_t)smem,
                                     st);
    vg_launch_counter++;
    vg_prof_end(VG_PROF_PAGG, st);
    if (e != cudaSuccess) {
        snprintf(g_jit_err, sizeof(g_jit_err), "pagg reduce launch: %s", cudaGetErrorString(e));
        return -1;
    }
    return 0;
}

// Compiles the reducer without launching it (no device needed).
int vgk_pagg_compile_only(const VgAggLaunch *L, const VgFinish *fin, int n_out, int G, int threads,
                          int *regs_out) {
    std::vector<char> cubin;
    int spill = 0;
    std::string log;
    const int rc = nvrtc_cubin(gen_pagg_source(*L, fin, n_out, G, threads, 1024 / threads), cubin, &spill, &log);
    snprintf(g_jit_err, sizeof(g_jit_err), "%s%.1800s", rc == 0 ? "" : "NVRTC failed:\n", log.c_str());
    if (regs_out) {
        const char *p = strstr(log.c_str(), "Used ");
        *regs_out = p ? atoi(p + 5) : -1;
    }
    return rc;
}

}  // extern "C"

// ---------------------------------------------------------------------
// self-test: generates and compiles representative plan shapes (no device
// needed).  Shape 0: left join + value*weight sum + n() keyed on a dense
// build-side attribute (direct-addressed payload copy); 1: filter (double and int64 ranges) + mean + n()
// over a selection vector; 2: two keys (int64, double), bool column, int64
// division, min / max / integer sum / count / bool min, first-seen order;
// 3: inner join on a coerced double key, build columns gathered by row;
// 4: shape 0 on a hashed join table; 5-7: partition mode (partitioned
// aggregation's first step) with per-CTA ranges, behind a filter, with
// global cursors.
// Returns 0 and the kernel's register count, or -1 (vgk_jit_error()).
// ---------------------------------------------------------------------
namespace {

VgOperand op_col(int side, int col, int type) {
    VgOperand o;
    memset(&o, 0, sizeof(o));
    o.side = side;
    o.col = col;
    o.type = type;
    return o;
}

VgValue val_plain(VgOperand a) {
    VgValue v;
    memset(&v, 0, sizeof(v));
    v.op = 0;
    v.type = a.type;
    v.a = a;
    return v;
}

VgValue val_op(int op, int type, VgOperand a, VgOperand b) {
    VgValue v;
    memset(&v, 0, sizeof(v));
    v.op = op;
    v.type = type;
    v.a = a;
    v.b = b;
    return v;
}

// Plans of the partitioned-aggregation self-tests (partition mode set).
void pagg_plan(VgAggLaunch &L, int variant) {
    static double dummy[4];
    memset(&L, 0, sizeof(L));
    L.part = 1;
    L.po.n_buckets = 2;
    L.cache_slots = 32;
    if (variant == 0) {
        L.n_pcols = 3;
        L.pcols[0] = VgCol{VEC_INT64, 0, dummy, nullptr};
        L.pcols[1] = VgCol{VEC_DOUBLE, 0, dummy, nullptr};
        L.pcols[2] = VgCol{VEC_INT64, 0, dummy, nullptr};
        L.n_keys = 1;
        L.key[0] = val_plain(op_col(VG_SIDE_PROBE, 0, VEC_INT64));
        L.n_accs = 4;
        L.acc[0].cls = VG_ACC_SUM_F64;
        L.acc[0].in = val_plain(op_col(VG_SIDE_PROBE, 1, VEC_DOUBLE));
        L.acc[1].cls = VG_ACC_MIN_I64;
        L.acc[1].in = val_plain(op_col(VG_SIDE_PROBE, 2, VEC_INT64));
        L.acc[2].cls = VG_ACC_MAX_I64;
        L.acc[2].in = val_plain(op_col(VG_SIDE_PROBE, 2, VEC_INT64));
        L.acc[3].cls = VG_ACC_COUNT_ALL;
    } else {
        L.n_pcols = 4;
        L.pcols[0] = VgCol{VEC_INT64, 0, dummy, nullptr};
        L.pcols[1] = VgCol{VEC_DOUBLE, 0, dummy, nullptr};
        L.pcols[2] = VgCol{VEC_INT64, 0, dummy, nullptr};
        L.pcols[3] = VgCol{VEC_BOOL, 0, dummy, nullptr};
        L.pred.n_terms = 1;
        L.pred.term[0] = VgTerm{1, VG_TERM_RANGE, VG_DOM_DOUBLE, 0, 0, 0};
        L.n_keys = 1;
        L.key[0] = val_plain(op_col(VG_SIDE_PROBE, 0, VEC_INT64));
        L.n_accs = 5;
        L.acc[0].cls = VG_ACC_SUM_I64;
        L.acc[0].in = val_plain(op_col(VG_SIDE_PROBE, 2, VEC_INT64));
        L.acc[1].cls = VG_ACC_MIN_F64;
        L.acc[1].na_rm = 1;
        L.acc[1].in = val_plain(op_col(VG_SIDE_PROBE, 1, VEC_DOUBLE));
        L.acc[2].cls = VG_ACC_MAX_F64;
        L.acc[2].in = val_op('*', VEC_DOUBLE, op_col(VG_SIDE_PROBE, 1, VEC_DOUBLE), op_col(VG_SIDE_PROBE, 2, VEC_INT64));
        L.acc[3].cls = VG_ACC_COUNT_VALID;
        L.acc[3].in = val_plain(op_col(VG_SIDE_PROBE, 1, VEC_DOUBLE));
        L.acc[4].cls = VG_ACC_NA_ONLY;
        L.acc[4].in = val_plain(op_col(VG_SIDE_PROBE, 3, VEC_BOOL));
    }
}

}  // namespace

namespace {

// The launches of the self-test shapes (no device memory behind them).
int selftest_plan(VgAggLaunch &L, int shape) {
    memset(&L, 0, sizeof(L));
    static double dummy[4];
    L.cache_slots = 1024;
    if (shape == 0 || shape == 4 || shape == 10 || shape == 11) {
        L.n_pcols = 2;
        L.pcols[0] = VgCol{VEC_INT64, 0, dummy, nullptr};
        L.pcols[1] = VgCol{VEC_DOUBLE, 0, dummy, nullptr};
        L.n_bcols = 2;
        L.bcols[0] = VgCol{VEC_INT64, 0, dummy, nullptr};
        L.bcols[1] = VgCol{VEC_DOUBLE, 0, dummy, nullptr};
        L.has_join = 1;
        L.join_kind = JOIN_LEFT;
        L.n_jkeys = 1;
        L.jkey_col[0] = 0;
        L.jt.cap = 64;
        L.jt.n_keys = 1;
        L.jt.key_types[0] = VEC_INT64;
        L.jt.slots = (VgJSlot *)dummy;
        L.n_keys = 1;
        L.key[0] = val_plain(op_col(VG_SIDE_BUILD, 0, VEC_INT64));
        L.n_accs = 2;
        L.acc[0].cls = VG_ACC_SUM_F64;
        L.acc[0].in = val_op('*', VEC_DOUBLE, op_col(VG_SIDE_PROBE, 1, VEC_DOUBLE), op_col(VG_SIDE_BUILD, 1, VEC_DOUBLE));
        L.acc[1].cls = VG_ACC_COUNT_ALL;
        L.skip_count_mask = 1u;
        L.dense = 1;
        L.dense_n = 256;
        L.jpay = (const VgJPay *)dummy;
        L.jpay_n = 2;
        L.jt.direct = shape != 4;   // shape 4: hashed table, linear-probing chain
        L.jt.dmin = 1;
        static uint32_t defer_dummy[4];
        L.defer_bits = defer_dummy;     // the dense cache defers rows to the replay kernel
        L.defer_n = defer_dummy + 2;
        L.defer_words = 1;
        if (shape == 11) {          // compact payload entries, the group key narrowed
            L.jpay16 = 1;
            L.jpay_narrow = 0;
        }
        if (shape == 10) {          // a filter on the probe side in front of the join
            L.pred.n_terms = 1;
            L.pred.term[0] = VgTerm{1, VG_TERM_RANGE, VG_DOM_DOUBLE, 0, 0, 0};
        }
    } else if (shape == 1 || shape == 8 || shape == 9) {
        // filter -> group_by -> sum, n: 1 behind a selection vector, 8 over
        // whole batches (passing rows queued per warp), 9 the same in
        // first-seen group order
        static int32_t sel[4];
        L.sel = shape == 1 ? sel : nullptr;
        L.track_first = shape == 9;
        L.n_pcols = 3;
        L.pcols[0] = VgCol{VEC_INT64, 0, dummy, nullptr};
        L.pcols[1] = VgCol{VEC_DOUBLE, 0, dummy, nullptr};
        L.pcols[2] = VgCol{VEC_INT64, 0, dummy, nullptr};
        L.pred.n_terms = 2;
        L.pred.term[0] = VgTerm{1, VG_TERM_RANGE, VG_DOM_DOUBLE, 0, 0, 0};
        L.pred.term[1] = VgTerm{2, VG_TERM_NOT_RANGE, VG_DOM_INT64, 0, 0, 0};
        L.n_keys = 1;
        L.key[0] = val_plain(op_col(VG_SIDE_PROBE, 0, VEC_INT64));
        L.n_accs = 2;
        L.acc[0].cls = VG_ACC_SUM_F64;
        L.acc[0].in = val_plain(op_col(VG_SIDE_PROBE, 1, VEC_DOUBLE));
        L.acc[1].cls = VG_ACC_COUNT_ALL;
    } else if (shape == 2) {
        L.n_pcols = 4;
        L.pcols[0] = VgCol{VEC_INT64, 0, dummy, nullptr};
        L.pcols[1] = VgCol{VEC_DOUBLE, 0, dummy, nullptr};
        L.pcols[2] = VgCol{VEC_BOOL, 0, dummy, nullptr};
        L.pcols[3] = VgCol{VEC_INT64, 0, dummy, nullptr};
        L.n_keys = 2;
        L.key[0] = val_plain(op_col(VG_SIDE_PROBE, 0, VEC_INT64));
        L.key[1] = val_plain(op_col(VG_SIDE_PROBE, 1, VEC_DOUBLE));
        L.n_accs = 5;
        L.acc[0].cls = VG_ACC_MIN_I64;
        L.acc[0].in = val_op('/', VEC_INT64, op_col(VG_SIDE_PROBE, 3, VEC_INT64), op_col(VG_SIDE_PROBE, 0, VEC_INT64));
        L.acc[1].cls = VG_ACC_MAX_F64;
        L.acc[1].na_rm = 1;
        L.acc[1].in = val_plain(op_col(VG_SIDE_PROBE, 1, VEC_DOUBLE));
        L.acc[2].cls = VG_ACC_SUM_I64;
        L.acc[2].in = val_op('%', VEC_INT64, op_col(VG_SIDE_PROBE, 3, VEC_INT64), op_col(VG_SIDE_LIT, 0, VEC_INT64));
        L.acc[2].in.b.lit = 7;
        L.acc[3].cls = VG_ACC_COUNT_VALID;
        L.acc[3].in = val_plain(op_col(VG_SIDE_PROBE, 1, VEC_DOUBLE));
        L.acc[4].cls = VG_ACC_NA_ONLY;
        L.acc[4].in = val_plain(op_col(VG_SIDE_PROBE, 2, VEC_BOOL));
        L.track_first = 1;
    } else if (shape == 3) {
        // inner join, build columns gathered by row (no payload copy), hashed cache
        L.n_pcols = 2;
        L.pcols[0] = VgCol{VEC_INT64, 0, dummy, nullptr};
        L.pcols[1] = VgCol{VEC_DOUBLE, 0, dummy, nullptr};
        L.n_bcols = 3;
        L.bcols[0] = VgCol{VEC_INT64, 0, dummy, nullptr};
        L.bcols[1] = VgCol{VEC_DOUBLE, 0, dummy, nullptr};
        L.bcols[2] = VgCol{VEC_BOOL, 0, dummy, nullptr};
        L.has_join = 1;
        L.join_kind = JOIN_INNER;
        L.n_jkeys = 1;
        L.jkey_col[0] = 0;
        L.jkey_conv[0] = 1;
        L.jt.cap = 64;
        L.jt.n_keys = 1;
        L.jt.key_types[0] = VEC_DOUBLE;
        L.jt.slots = (VgJSlot *)dummy;
        L.n_keys = 2;
        L.key[0] = val_plain(op_col(VG_SIDE_BUILD, 0, VEC_INT64));
        L.key[1] = val_plain(op_col(VG_SIDE_BUILD, 2, VEC_BOOL));
        L.n_accs = 2;
        L.acc[0].cls = VG_ACC_SUM_F64;
        L.acc[0].in = val_op('-', VEC_DOUBLE, op_col(VG_SIDE_PROBE, 1, VEC_DOUBLE), op_col(VG_SIDE_BUILD, 1, VEC_DOUBLE));
        L.acc[1].cls = VG_ACC_MAX_I64;
        L.acc[1].in = val_plain(op_col(VG_SIDE_BUILD, 0, VEC_INT64));
        L.track_first = 1;
    } else if (shape >= 5 && shape <= 7) {
        // partition mode of group_by(key) |> summarise(sum(x), mean(x), min(y), max(y), n()): 5 per-CTA
        // record ranges, 6 the same behind a filter (holes), 7 global cursors
        pagg_plan(L, shape == 6 ? 1 : 0);
        if (shape != 7) L.po.cta_off = (const uint64_t *)dummy;
    } else {
        snprintf(g_jit_err, sizeof(g_jit_err), "no such self-test shape %d", shape);
        return -1;
    }
    return 0;
}

}  // namespace

extern "C" int vgpu_jit_selftest(int shape, int *regs) {
    static VgAggLaunch L;
    if (selftest_plan(L, shape) != 0) return -1;
    return vgk_agg_jit_compile_only(&L, regs);
}

// The launch signature's premise, checked on a self-test shape (no device
// needed): every field the signature reduces -- pointers to set / unset,
// per-batch numbers -- changed to other values leaves the signature and
// the generated source unchanged.  Returns 0, or 1 on a mismatch.
extern "C" int vgpu_jit_sigcheck(int shape) {
    static VgAggLaunch L, M;
    if (selftest_plan(L, shape) != 0) return -1;
    const int S = vgk_agg_jit_slots(&L);
    const bool vec = vec_ok(L);
    const Shape sh = plan_shape(L);
    const std::string sig = launch_signature(L, S, vec, sh), src = gen_source(L, S, vec, sh);
    for (int v = 1; v <= 3; v++) {
        memcpy(&M, &L, sizeof(M));
        // another non-NULL value for every pointer that is set (256-byte
        // aligned, as device allocations are), NULL ones left NULL
        const uintptr_t other = (uintptr_t)4096 * (uintptr_t)(v * 7919);
        auto move = [&](auto *&ptr) { shift_ptr(ptr, other); };
        move(M.sel);
        for (int i = 0; i < VG_MAX_COLS; i++) {
            move(M.pcols[i].data);
            move(M.pcols[i].valid);
            move(M.bcols[i].data);
            move(M.bcols[i].valid);
        }
        move(M.jt.slots); move(M.jt.state); move(M.jt.keys); move(M.jt.start); move(M.jt.count); move(M.jt.rows);
        move(M.jt.err);
        move(M.gt.state); move(M.gt.nullmask); move(M.gt.keys); move(M.gt.first_row); move(M.gt.n_used);
        move(M.gt.err);
        for (int a = 0; a < VG_MAX_ACCS; a++) {
            move(M.gt.cnt[a]); move(M.gt.val[a]); move(M.gt.flags[a]); move(M.gt.lacc[a]);
        }
        move(M.spill_rows); move(M.spill_rows_n); move(M.spill_cache); move(M.spill_cache_n); move(M.jpay);
        move(M.po.rec); move(M.po.cursor); move(M.po.end); move(M.po.err); move(M.po.cta_off); move(M.po.start);
        move(M.defer_bits); move(M.defer_n);
        M.n_rows = 1000003 * v;
        M.sel_n = 77 * v;
        M.row_base = 123456789ll * v;
        M.batch_idx = 5 * v;
        M.li_base = 4096 * v;
        M.spill_rows_cap = 65536 * v;
        M.spill_cache_cap = 1024 * v;
        M.dense_min = -17 * v;
        M.jpay_min = 3 * v;
        M.jt.cap = 1 << (10 + v);
        M.jt.dmin = 9 * v;
        M.jt.n_build = 999 * v;
        M.gt.cap = 1 << (12 + v);
        M.po.omin = 11ull * (uint64_t)v;
        M.po.shift = 3 + v;
        M.po.n_buckets = 16 << v;
        M.po.total = 1000ull * (uint64_t)v;
        M.defer_words = 100 * v;
        const int S2 = vgk_agg_jit_slots(&M);
        const bool vec2 = vec_ok(M);
        const Shape sh2 = plan_shape(M);
        if (S2 != S || vec2 != vec) return 1;
        if (launch_signature(M, S2, vec2, sh2) != sig) return 1;
        if (gen_source(M, S2, vec2, sh2) != src) return 1;
    }
    return 0;
}

// Partitioned-aggregation reducer of representative plans (no device
// needed): 0, the 5-aggregate high-cardinality plan; 1, every accumulator
// class (int64 sum, double min / max with na.rm, count of valid values,
// bool min) with a filter in front.  Returns 0 and the register count, or
// -1 (vgk_jit_error()).
extern "C" int vgpu_pagg_selftest(int shape, int *regs) {
    static VgAggLaunch L;
    VgFinish fin[VG_MAX_OUTS];
    int n_out = 0;
    memset(fin, 0, sizeof(fin));
    // shapes 2 and 3: the plans of 0 and 1 for two reducer CTAs per SM;
    // 4 and 5 for four, 6 and 7 for eight
    const int ctas = shape >= 6 ? 8 : shape >= 4 ? 4 : shape >= 2 ? 2 : 1;
    shape %= 2;
    if (shape == 0) {
        pagg_plan(L, 0);
        const int kinds[5] = {AGG_SUM, AGG_MEAN, AGG_MIN, AGG_MAX, AGG_COUNT_STAR};
        const int accs[5] = {0, 0, 1, 2, 3};
        const int types[5] = {VEC_DOUBLE, VEC_DOUBLE, VEC_INT64, VEC_INT64, VEC_INT64};
        for (int o = 0; o < 5; o++) fin[o] = VgFinish{accs[o], kinds[o], types[o], 0};
        n_out = 5;
    } else if (shape == 1) {
        pagg_plan(L, 1);
        fin[0] = VgFinish{0, AGG_SUM, VEC_INT64, 0};
        fin[1] = VgFinish{0, AGG_MEAN, VEC_INT64, 0};
        fin[2] = VgFinish{1, AGG_MIN, VEC_DOUBLE, 1};
        fin[3] = VgFinish{2, AGG_MAX, VEC_DOUBLE, 0};
        fin[4] = VgFinish{3, AGG_COUNT, VEC_DOUBLE, 0};
        fin[5] = VgFinish{4, AGG_MIN, VEC_BOOL, 0};
        n_out = 6;
    } else {
        snprintf(g_jit_err, sizeof(g_jit_err), "no such self-test shape %d", shape);
        return -1;
    }
    const int G = vgk_pagg_groups_for(&L, ctas);
    if (G <= 0) {
        snprintf(g_jit_err, sizeof(g_jit_err), "plan does not fit the reducer");
        return -1;
    }
    return vgk_pagg_compile_only(&L, fin, n_out, G, 1024 / ctas, regs);
}

// Host check of the 32-bit digit split against the 64-bit one on n bit
// patterns (edge cases first, then a xorshift sequence from seed):
// returns the number of mismatches.
extern "C" long long vgk_digits_selftest(long long n, unsigned long long seed) {
    const uint64_t edge[] = {0ull, 0x8000000000000000ull, 1ull, 0x8000000000000001ull, 0x000FFFFFFFFFFFFFull,
                             0x0010000000000000ull, 0x3FF0000000000000ull, 0xBFF0000000000000ull,
                             0x7FEFFFFFFFFFFFFFull, 0xFFEFFFFFFFFFFFFFull, 0x7FF0000000000000ull,
                             0xFFF0000000000000ull, 0x7FF8000000000000ull, 0x7FF0000000000001ull,
                             0x4330000000000000ull, 0x433FFFFFFFFFFFFFull, 0x0000000100000000ull};
    long long bad = 0;
    uint64_t x = seed | 1;
    for (long long i = 0; i < n; i++) {
        uint64_t b;
        if (i < (long long)(sizeof(edge) / sizeof(edge[0]))) {
            b = edge[i];
        } else {
            x ^= x << 13; x ^= x >> 7; x ^= x << 17;
            b = x;
        }
        const VgDigits r = vg_split_double(b);
        const VgDigits32 q = vg_split_double32(b);
        if (r.special != q.special) { bad++; continue; }
        if (r.special) continue;
        if ((r.lo < 0) != (q.zero != 0)) { bad++; continue; }
        if (r.lo < 0) continue;
        const int64_t s = q.neg ? -1 : 1;
        if (r.lo != q.word || r.d0 != s * (int64_t)q.d0 || r.d1 != s * (int64_t)q.d1 || r.d2 != s * (int64_t)q.d2)
            bad++;
    }
    return bad;
}
