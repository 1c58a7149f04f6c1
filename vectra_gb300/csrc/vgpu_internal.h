/*
 * vgpu_internal.h -- the contract between libvgpu's C11 host layer
 * (nodes, plan compilation, memory) and its sm_103a CUDA kernels.
 *
 * Plain C structs only: the host side fills them, the .cu side launches
 * kernels with them passed by value.
 */
#ifndef VGPU_INTERNAL_H
#define VGPU_INTERNAL_H

#ifdef __CUDACC_RTC__
#include "vg_rtc_types.h"
#else
#include <stdint.h>
#include <stddef.h>
#endif
#include "vectra_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *vg_stream_t;

/* ------------------------------------------------------------------ */
/* device column views                                                 */
/* ------------------------------------------------------------------ */

/* One column resident in device memory.  data: 8-byte values for int64 and
 * double, one byte per row for bool.  valid: the column's validity bitmap
 * read as little-endian 32-bit words (bit i%32 of word i/32 == bit i%8 of
 * byte i/8 of the host bitmap); NULL means every row is valid. */
typedef struct {
    int32_t type;              /* VecType */
    int32_t voff;              /* bit offset of row 0 within valid[0] (0..31) */
    const void *data;
    const uint32_t *valid;
} VgCol;

/* A string value on the device: its length, its first four bytes packed
 * big-endian and zero-padded (two prefixes compare as the strings do, so
 * most comparisons end there), and a pointer to its bytes.  A VEC_STRING
 * column's data is one view per row; the bytes live in the batch's own
 * device block (or a dictionary's arena). */
typedef struct {
    uint32_t len;
    uint32_t pre;
    const char *ptr;
} VgStrView;

#define VG_MAX_COLS   24
#define VG_MAX_TERMS  12
#define VG_MAX_KEYS   4
#define VG_MAX_ACCS   12   /* distinct accumulators per group-agg */
#define VG_MAX_OUTS   32   /* aggregate outputs per group-agg */
#define VG_MAX_INSNS  48

/* ------------------------------------------------------------------ */
/* predicates                                                          */
/* ------------------------------------------------------------------ */

/* A conjunction of column-vs-constant terms, each folded on the host into
 * an inclusive range in the column's integer domain (int64 value, bool
 * byte, or the order-preserving integer image of a double).  A row is kept
 * iff every term keeps it; NA rows of a compared column are dropped, which
 * is what Kleene AND followed by `valid && true` does (src/filter.c:20). */
enum {
    VG_TERM_RANGE = 0,       /* keep iff valid && lo <= v <= hi            */
    VG_TERM_NOT_RANGE = 1,   /* keep iff valid && !(lo <= v <= hi)         */
    VG_TERM_IS_NA = 2,       /* keep iff !valid                            */
    VG_TERM_NOT_NA = 3,      /* keep iff valid                             */
    VG_TERM_NONE = 4         /* keep nothing (FALSE or NA literal)         */
};
enum { VG_DOM_INT64 = 0, VG_DOM_DOUBLE = 1, VG_DOM_BOOL = 2 };

typedef struct {
    int32_t col;             /* index into the launch's column table */
    int32_t kind;            /* VG_TERM_* */
    int32_t domain;          /* VG_DOM_* */
    int32_t nan_keep;        /* double domain: keep a valid NaN row? */
    int64_t lo, hi;
} VgTerm;

typedef struct {
    int32_t n_terms;
    int32_t pad;
    VgTerm term[VG_MAX_TERMS];
} VgPred;

/* ------------------------------------------------------------------ */
/* general expressions (postfix programs)                              */
/* ------------------------------------------------------------------ */

/* Stack machine over (64-bit payload, valid) cells.  Each instruction
 * leaves a value of a statically known type; coercions are explicit. */
enum {
    VI_COL_I64 = 1,   /* push column a as int64            */
    VI_COL_F64,       /* push column a as double           */
    VI_COL_BOOL,      /* push column a as bool (0/1)       */
    VI_LIT_I64,       /* push imm                          */
    VI_LIT_F64,       /* push imm (bit pattern of double)  */
    VI_LIT_BOOL,      /* push imm (0/1)                    */
    VI_LIT_NA,        /* push NA                           */
    VI_I2F,           /* top: int64 -> double              */
    VI_ARITH_I64,     /* a = op char                       */
    VI_ARITH_F64,
    VI_CMP_I64,       /* a = cmp code (VG_CMP_*)           */
    VI_CMP_F64,
    VI_AND,
    VI_OR,
    VI_NOT,
    VI_IS_NA,
    VI_NEG_I64,
    VI_NEG_F64,
    /* strings: a string cell holds a pointer to its bytes and its length */
    VI_COL_STR,       /* push column a (string views)      */
    VI_LIT_STR,       /* push pool bytes [imm, imm + a)    */
    VI_CMP_STR,       /* a = cmp code: memcmp, then length */
    VI_NCHAR,         /* top: string -> int64 byte count   */
    VI_SUBSTR,        /* (s, start, stop) -> substring     */
    VI_GREPL,         /* top: string -> contains pool bytes [imm, imm + a) */
    VI_F2I            /* top: double -> int64, toward zero */
};
#define VG_PROG_POOL 512   /* bytes of string literals per program */
enum { VG_CMP_EQ = 0, VG_CMP_NE, VG_CMP_LT, VG_CMP_LE, VG_CMP_GT, VG_CMP_GE };

typedef struct {
    int32_t op;
    int32_t a;
    int64_t imm;
} VgInsn;

typedef struct {
    int32_t n;
    int32_t result_type;     /* VecType of the value left on the stack */
    int32_t max_depth;
    int32_t pool_n;          /* bytes of pool in use */
    VgInsn insn[VG_MAX_INSNS];
    char pool[VG_PROG_POOL]; /* string literals (no terminators) */
} VgProg;

/* ------------------------------------------------------------------ */
/* values read by fused kernels                                        */
/* ------------------------------------------------------------------ */

/* An operand is a column of the probe (or only) side, a column of the
 * build side of a join (NA for unmatched LEFT rows), or a constant. */
enum { VG_SIDE_PROBE = 0, VG_SIDE_BUILD = 1, VG_SIDE_LIT = 2, VG_SIDE_NA = 3 };

typedef struct {
    int32_t side;
    int32_t col;
    int32_t type;            /* VecType of the operand */
    int32_t pad;
    int64_t lit;             /* literal payload (int64 or double bits) */
} VgOperand;

/* value = a, or (a op b) with the reference's arithmetic rules
 * (src/scalar_ops.c:11-66): computed in `type` (int64 or double) after
 * coercing both operands; int64 division/modulo by zero is NA. */
typedef struct {
    int32_t op;              /* 0 = plain operand, else '+','-','*','/','%' */
    int32_t type;            /* result VecType */
    VgOperand a, b;
} VgValue;

/* ------------------------------------------------------------------ */
/* grouped aggregation                                                 */
/* ------------------------------------------------------------------ */

/* Accumulator classes; aggregate outputs are derived from them at finish
 * (every output is double, src/group_agg.c:658-661). */
enum {
    VG_ACC_COUNT_ALL = 0,    /* n()                                      */
    VG_ACC_COUNT_VALID,      /* count of non-NA values                   */
    VG_ACC_SUM_I64,          /* int64 / bool sum (wrapping), count, NA   */
    VG_ACC_SUM_F64,          /* exact fixed-point double sum, count, NA  */
    VG_ACC_MIN_I64,
    VG_ACC_MAX_I64,
    VG_ACC_MIN_F64,          /* on the ordered-integer image             */
    VG_ACC_MAX_F64,
    VG_ACC_NA_ONLY           /* min/max of bool: only NA poisoning       */
};

typedef struct {
    int32_t cls;             /* VG_ACC_* */
    int32_t na_rm;
    VgValue in;
} VgAccSpec;

/* Global group table.  Slots are claimed with a CAS on state
 * (0 empty, 1 being written, 2 ready); keys are normalised 64-bit words
 * (double -0 folded to +0) plus a per-slot NA mask. */
#define VG_LACC_WORDS 66     /* 32-bit digits of a full-range double sum */

/* kernel error bits (group / join tables) */
#define VG_ERR_WAIT   1u     /* a bounded wait expired */
#define VG_ERR_FULL   2u     /* a table or spill list was full */
#define VG_ERR_PROG   4u     /* malformed expression program */
#define VG_ERR_SPILL  8u     /* a spill list overflowed */

typedef struct {
    int64_t   cap;           /* power of two */
    uint32_t *state;
    uint32_t *nullmask;
    uint64_t *keys;          /* [VG_MAX_KEYS][cap] */
    uint64_t *first_row;     /* min global row id of each group */
    /* per accumulator (index a): */
    uint64_t *cnt[VG_MAX_ACCS];    /* count (valid values, or all rows) */
    int64_t  *val[VG_MAX_ACCS];    /* int64 sum / min / max, or ordered image */
    uint32_t *flags[VG_MAX_ACCS];  /* bit0 has_na, bit1 has_value, bit2 NaN, bit3 +inf, bit4 -inf */
    int64_t  *lacc[VG_MAX_ACCS];   /* [cap][VG_LACC_WORDS] digit words */
    uint32_t *n_used;        /* number of occupied slots */
    uint32_t *err;           /* error word: nonzero = a bounded wait expired / table full */
} VgGroupTable;

/* A string dictionary: every distinct string gets the next int64 code and
 * a copy of its bytes in the arena; slot[] is an open-addressing table of
 * codes (0xFFFFFFFF empty, 0xFFFFFFFE being filled).  The host keeps
 * room for every row of a launch before it (table at most half full). */
#define VG_DICT_CODES  0     /* ctr[]: codes given out */
#define VG_DICT_USED   1     /*        arena bytes used */
#define VG_DICT_ROWS   2     /*        pre-pass: valid rows of the batch */
#define VG_DICT_BYTES  3     /*        pre-pass: their bytes */
#define VG_DICT_MAXLEN 4     /*        longest string seen */
#define VG_DICT_CTRS   8
typedef struct {
    int64_t   cap;           /* slots, power of two */
    uint32_t *slot;
    int64_t   codes_cap;
    uint64_t *c_hash;
    int64_t  *c_off;
    uint32_t *c_len;
    char     *arena;
    int64_t   arena_cap;
    unsigned long long *ctr; /* VG_DICT_CTRS counters */
} VgStrDict;

/* Build-row payload inlined into a copy of a single-key join table's
 * slots (same capacity and slot positions): one 32-byte sector per probe
 * gives the key, the build row and up to two build columns with their
 * validity.  Built only for unique build keys. */
typedef struct {
    uint64_t key;
    int32_t  start;          /* build row */
    uint32_t meta;           /* bit0: key present; bit 1+c: payload column c valid */
    uint64_t p[2];
} VgJPay;

/* The compact form of the payload copy of a direct-addressed table (the
 * slot is key - min, so no key; the fused aggregation reads no build row):
 * 16 bytes per slot.  `a` holds the one payload column that is not
 * narrowed (any type); `b` the narrowed one: an int64 column whose valid
 * values span less than 2^32 as (value - its minimum), a bool column as its
 * byte.  meta as in VgJPay.  Used when the payload is one column, or two of
 * which one narrows. */
typedef struct {
    uint64_t a;
    uint32_t b;
    uint32_t meta;
} VgJPay16;

/* Join hash table over the build side (keys unique per slot; rows of a key
 * listed in ascending build-row order in rows[start .. start+count)). */
/* Single-key join slot: one 16-byte sector per probe.  key == VG_JEMPTY
 * marks a free slot; the one key equal to that marker (if any) lives in
 * the extra slot at index cap. */
typedef struct {
    uint64_t key;
    int32_t  start;
    int32_t  count;
} VgJSlot;
#define VG_JEMPTY 0x8000000000000000ull

typedef struct {
    int64_t   cap;           /* power of two (hashed) or the key range (direct) */
    int32_t   n_keys;
    int32_t   key_types[VG_MAX_KEYS];
    /* Direct addressing for one int64 key whose build values span a range
     * comparable to the build row count (surrogate / dense ids): the slot
     * of key k is k - dmin for k in [dmin, dmin + cap), no hashing, one
     * slot read per probe, presence = count > 0. */
    int32_t   direct;
    int32_t   pad_direct;
    int64_t   dmin;
    VgJSlot  *slots;         /* single-key tables: cap + 1 slots */
    uint32_t *state;         /* composite-key tables: slot locks ... */
    uint64_t *keys;          /* ... [n_keys][cap] key words ... */
    int32_t  *start;         /* ... first position in rows ... */
    int32_t  *count;         /* ... rows with this key */
    int32_t  *rows;          /* n_build entries, or NULL when keys are unique */
    int64_t   n_build;
    uint32_t *err;
} VgJoinTable;

/* Partitioned aggregation (many groups, one int64 key, key-ordered
 * output): the fused kernel writes every row with a valid key as a record
 * into the key-range bucket of its key, instead of updating a table.
 * Record (rec_words 64-bit words): key, validity bits of the values, the
 * plan's distinct aggregate input values.  Bucket of key k:
 * min(n_buckets - 1, max(0, (k ^ 2^63) - omin) >> shift); bucket b's
 * records go to [start[b], end[b]) through its cursor. */
typedef struct {
    uint64_t *rec;
    unsigned long long *cursor;   /* per bucket (stride VG_PAGG_CURSOR_STRIDE): next record position */
    const uint64_t *end;          /* per bucket: one past its last position */
    uint64_t omin;
    int32_t shift;
    int32_t n_buckets;
    int32_t rec_words;
    int32_t n_vals;
    uint32_t *err;                /* VG_ERR_FULL: a bucket range was exceeded */
    /* Per-CTA ranges (cta_off != NULL): CTA c of the launch owns records
     * [cta_off[b * grid + c], cta_off[b * grid + c + 1]) of bucket b,
     * counted beforehand over exactly the rows it processes, and hands
     * them out with shared-memory counters instead of the global cursors;
     * positions it leaves unused (rows a filter or inner join dropped)
     * are written as holes.  start[b]: bucket b's first position. */
    const uint64_t *cta_off;
    const uint64_t *start;
    uint64_t total;               /* records of the region (no position at or past it is written) */
} VgPartOut;

/* flags word of a partition record that is a hole (no row) */
#define VG_PAGG_HOLE 0x8000000000000000ull

#define VG_PAGG_MAX_REGIONS 64
/* the partition pass's bucket cursors are VgPartOut.cursor[b * stride]: one
 * per 128-byte line, so cursor atomics of different buckets do not queue
 * on the same line */
#define VG_PAGG_CURSOR_STRIDE 16
/* most buckets whose per-CTA counters fit in the partition kernel's shared memory */
#define VG_PAGG_CTA_BUCKETS 32768

/* Second step of the partitioned aggregation: one CTA per bucket at a
 * time (bucket order from a ticket) aggregates the bucket's records in
 * shared memory, orders its groups by key and writes their results to
 * the staging area at stage_off[b].  Records of bucket b in region r:
 * [roff[r][b], rend[r][b]). */
typedef struct {
    int32_t n_regions;
    int32_t n_buckets;            /* buckets [bucket_base, bucket_base + n_buckets) */
    int32_t rec_words;
    int32_t n_out;
    int32_t bucket_base;
    int32_t pad_base;
    uint64_t omin;                /* bucket b holds the order words [omin + (b << shift), +2^shift) */
    int32_t shift;
    int32_t pad_shift;
    const uint64_t *rec[VG_PAGG_MAX_REGIONS];
    const uint64_t *roff[VG_PAGG_MAX_REGIONS];
    const unsigned long long *rend[VG_PAGG_MAX_REGIONS];
    const uint64_t *stage_off;
    uint32_t *gc;                 /* per bucket: groups written */
    uint32_t *ovf;                /* per bucket: 1 = more groups than one CTA holds (nothing written) */
    unsigned int *ticket;
    uint64_t *st_key;
    uint32_t *st_ok;              /* bit o: output o is valid */
    double *st_out[VG_MAX_OUTS];
    double *fs[VG_MAX_ACCS];      /* compensated fallback of double sums, per staging position */
    double *fc[VG_MAX_ACCS];
    uint32_t *warn;
    uint32_t *err;
} VgPaggReduce;

/* One fused aggregation launch over a batch of rows:
 *   rows -> [predicate] -> [join probe, per match] -> group keys / values
 *   -> per-CTA shared-memory cache -> global group table. */
typedef struct {
    int64_t n_rows;              /* physical rows of the probe batch */
    const int32_t *sel;          /* optional selection vector (device) */
    int64_t sel_n;
    int64_t row_base;            /* global id of physical row 0 */
    int32_t n_pcols, n_bcols;
    VgCol pcols[VG_MAX_COLS];
    VgCol bcols[VG_MAX_COLS];
    VgPred pred;
    /* join */
    int32_t has_join;
    int32_t join_kind;           /* JOIN_INNER or JOIN_LEFT */
    int32_t n_jkeys;
    int32_t jkey_col[VG_MAX_KEYS];   /* probe columns */
    int32_t jkey_conv[VG_MAX_KEYS];  /* 1: probe int64/bool -> double to match a double build key */
    VgJoinTable jt;
    /* grouping */
    int32_t n_keys;
    int32_t n_accs;
    VgValue key[VG_MAX_KEYS];
    VgAccSpec acc[VG_MAX_ACCS];
    int32_t track_first;         /* record first-seen row per group */
    int32_t cache_slots;         /* power of two, 0 = no shared-memory cache */
    VgGroupTable gt;
    /* When the global table is full, work is spilled instead of dropped:
     * rows as (logical row, match << 8 | (acc + 1)) pairs (acc + 1 == 0:
     * every accumulator), shared-cache entries in a cache-layout area with
     * stride spill_cache_cap.  The host grows the table and replays both. */
    int64_t  *spill_rows;
    uint32_t *spill_rows_n;
    int64_t   spill_rows_cap;
    char     *spill_cache;
    uint32_t *spill_cache_n;
    int64_t   spill_cache_cap;
    const int64_t *replay;       /* replay list (pairs as above) or NULL */
    int64_t   replay_n;
    int64_t   batch_idx;         /* probe batch number (join ordering key) */
    int64_t   li_base;           /* logical offset of this launch's rows within the probe batch */
    /* Direct-mapped cache for a single int64 key known to lie in
     * [dense_min, dense_min + dense_n) (a build-side attribute): cache slot
     * = key - dense_min, slot dense_n holds the NA key.  0 = hashed cache. */
    int32_t   dense;
    int32_t   dense_n;
    int64_t   dense_min;
    /* Accumulators whose count no output reads (a SUM without MEAN). */
    uint32_t  skip_count_mask;
    /* Optional payload copy of the join table holding bcols[0..jpay_n)
     * (read by the run-time specialised kernel). */
    const VgJPay *jpay;
    int32_t   jpay_n;
    /* 1: jpay holds VgJPay16 entries; jpay_narrow: the payload column kept in
     * VgJPay16.b (-1: none, one payload column), jpay_min its minimum */
    int32_t   jpay16;
    int32_t   jpay_narrow;
    int64_t   jpay_min;
    /* 1: partitioned aggregation's first step (run-time specialised kernel
     * only): rows with a valid key become records (po); NA-key rows update
     * the group table gt, which holds the NA group alone. */
    int32_t   part;
    VgPartOut po;
    /* Dense cache, run-time specialised kernel: rows whose double sums fall
     * outside the CTA's digit window are deferred instead of updating the
     * global table in the row loop: bit li of word array f (one array of
     * defer_words words per double-sum accumulator, in accumulator order)
     * marks row li for accumulator f, defer_n counts the marks, and the
     * replay kernel that follows each launch applies them and clears them. */
    uint32_t *defer_bits;
    int64_t   defer_words;
    uint32_t *defer_n;
} VgAggLaunch;

/* ------------------------------------------------------------------ */
/* kernel entry points (implemented in the .cu files)                  */
/* ------------------------------------------------------------------ */

#ifndef __CUDACC_RTC__
int  vgk_num_sms(void);
const char *vgk_last_cuda_error(void);

/* filter: keep mask + selection vector over logical rows */
int vgk_filter_pred(const VgCol *cols, int n_cols, const VgPred *pred,
                    int64_t n_rows, const int32_t *d_sel_in, int64_t sel_n,
                    int32_t *d_sel_out, int64_t *h_count, void *d_scratch,
                    size_t scratch_bytes, vg_stream_t s);
int vgk_filter_prog(const VgCol *cols, int n_cols, const VgProg *prog,
                    int64_t n_rows, const int32_t *d_sel_in, int64_t sel_n,
                    int32_t *d_sel_out, int64_t *h_count, void *d_scratch,
                    size_t scratch_bytes, vg_stream_t s);
size_t vgk_filter_scratch_bytes(int64_t n_logical);

/* evaluate a program over logical rows into a dense output column */
int vgk_eval_prog(const VgCol *cols, int n_cols, const VgProg *prog,
                  int64_t n_rows, const int32_t *d_sel, int64_t sel_n,
                  void *d_out, uint32_t *d_out_valid, vg_stream_t s);

/* gather logical rows of a column into dense output (values + validity) */
int vgk_gather(const VgCol *col, const int32_t *d_idx, int64_t n_out,
               int null_if_negative, void *d_out, uint32_t *d_out_valid,
               vg_stream_t s);

/* gather n values into rows [row0, row0+n) of an existing column whose
 * validity words are zeroed beforehand (any row0; bits are OR-ed in) */
int vgk_gather_into(const VgCol *col, const int32_t *d_idx, int64_t n, void *d_out,
                    uint32_t *d_out_valid, int64_t row0, vg_stream_t s);

/* min (out[0]), max (out[1]) and count (out[2]) of the valid values of an
 * int64 column of n rows; d_out: 24 bytes of device scratch, h_out: host */
int vgk_col_minmax_i64(const VgCol *col, int64_t n, int64_t *d_out, int64_t *h_out, vg_stream_t s);

/* group table */
int vgk_group_table_init(VgGroupTable *gt, int n_keys, const int32_t *acc_cls,
                         int n_accs, vg_stream_t s);
int vgk_agg_launch(const VgAggLaunch *L, vg_stream_t s);
size_t vgk_agg_smem_bytes(const VgAggLaunch *L);
/* per occupied slot: compact slot ids (in slot order) into d_slots */
int vgk_group_table_compact(const VgGroupTable *gt, int32_t *d_slots,
                            uint32_t *h_n, vg_stream_t s);
/* results for the listed slots: keys + one double column per output */
typedef struct {
    int32_t acc;             /* accumulator index */
    int32_t finish;          /* AggKind of the output */
    int32_t in_type;         /* VecType of the aggregated input */
    int32_t na_rm;
} VgFinish;
int vgk_group_finish(const VgGroupTable *gt, int n_keys, const int32_t *key_types,
                     const int32_t *d_slots, int64_t n_groups,
                     const VgFinish *fin, int n_out,
                     uint64_t **d_key_out, uint32_t **d_key_valid,
                     double **d_out, uint32_t **d_out_valid,
                     uint32_t *d_warn, vg_stream_t s);
/* order slots: mode 0 = keys ascending (NA last), 1 = first-seen row */
int vgk_order_groups(const VgGroupTable *gt, int n_keys, const int32_t *key_types,
                     int32_t *d_slots, int64_t n_groups, int mode,
                     void *d_scratch, size_t scratch_bytes, vg_stream_t s);
size_t vgk_order_scratch_bytes(int64_t n_groups);

/* join */
int64_t vgk_join_cap(int64_t n_build);
size_t vgk_join_build_scratch_bytes(int64_t n_build);
/* pay (optional, (cap + 1) 32-byte entries of room): filled with the
 * payload copy of pay_cols[0..n_pay) when every key is unique (for direct
 * tables in passes of their own, which then also report min, max and count
 * of the valid values of int64 payload columns in h_pay_mm[3 c .. 3 c + 2],
 * and leave the slot table unfilled: *slots_ready == 0).  Direct tables
 * write VgJPay16 entries when the payload fits them: *h_pay_layout = -1
 * (one payload column) or the index of the narrowed column (its minimum in
 * *h_pay_min); -2: VgJPay entries. */
int vgk_join_build(VgJoinTable *jt, const VgCol *keys, int n_keys, const int32_t *key_conv,
                   int64_t n_build, void *d_scratch, size_t scratch_bytes, int64_t *h_distinct,
                   int64_t *h_maxdup, const VgCol *pay_cols, int n_pay, VgJPay *pay, int64_t *h_pay_mm,
                   int *h_pay_layout, int64_t *h_pay_min, int *slots_ready, vg_stream_t s);
/* fills the slot table of a unique-key direct table from its payload copy
 * (a build that returned *slots_ready == 0 with VgJPay entries) */
int vgk_join_slots_from_payload(const VgJoinTable *jt, const VgJPay *pay, vg_stream_t s);
/* the same from the key column itself (a build that wrote VgJPay16 entries,
 * which hold neither keys nor build rows); d_scratch: n_build * 4 + 256
 * bytes */
int vgk_join_slots_from_keys(const VgJoinTable *jt, const VgCol *key, int32_t key_conv, int64_t n_build,
                             void *d_scratch, vg_stream_t s);
size_t vgk_join_probe_scratch_bytes(int64_t n_logical);
int vgk_join_probe_count(const VgJoinTable *jt, const VgCol *pkeys, int n_keys, const int32_t *key_conv,
                         int64_t n_rows, const int32_t *d_sel, int64_t sel_n, int kind,
                         void *d_scratch, size_t scratch_bytes, int64_t *h_total, vg_stream_t s);
int vgk_join_probe_emit(const VgJoinTable *jt, int64_t n_rows, const int32_t *d_sel, int64_t sel_n,
                        int kind, void *d_scratch, size_t scratch_bytes, int32_t *d_out_probe,
                        int32_t *d_out_build, uint32_t *d_build_matched, vg_stream_t s);
int vgk_join_unmatched_build(const uint32_t *d_matched, int64_t n_build, int32_t *d_out, int64_t *h_n,
                             void *d_scratch, size_t scratch_bytes, vg_stream_t s);
const char *vgk_join_last_error(void);

/* strings (k_strings.cu) */
const char *vgk_str_last_error(void);
/* views of n rows in the reference's layout (offsets n + 1, bytes; the
 * first byte of d_bytes is the one at offset base) */
int vgk_str_views(const int64_t *d_offs, int64_t base, const char *d_bytes, int64_t n, VgStrView *d_out,
                  vg_stream_t s);
/* lengths of rows d_idx[j] (or j; NA and negative ids: 0) and, d_valid
 * given, the validity words of the packed column */
int vgk_str_lengths(const VgCol *c, const int32_t *d_idx, int64_t n, int32_t *d_len, uint32_t *d_valid,
                    vg_stream_t s);
/* their bytes to d_out + d_offs[j] */
int vgk_str_pack(const VgCol *c, const int32_t *d_idx, int64_t n, const int64_t *d_offs, char *d_out,
                 vg_stream_t s);
int vgk_dict_prepass(const VgCol *c, const int32_t *d_sel, int64_t n_logical, unsigned long long *d_ctr,
                     vg_stream_t s);
/* d_codes[p] of the logical rows p: the string's code (insert: new strings
 * get codes; otherwise -1 for a string not present); NA rows: 0 */
int vgk_dict_encode(const VgStrDict *d, const VgCol *c, const int32_t *d_sel, int64_t n_logical, int insert,
                    int64_t *d_codes, uint32_t *d_err, vg_stream_t s);
int vgk_dict_rehash(const VgStrDict *d, int64_t n_codes, uint32_t *d_err, vg_stream_t s);
/* views of the strings of d_codes[j] (through d_map when given) */
int vgk_dict_views(const VgStrDict *d, const int64_t *d_codes, const uint32_t *d_valid, const int32_t *d_map,
                   int64_t n, VgStrView *d_out, vg_stream_t s);
/* (n_chunks + 1) int64 columns of n_codes rows whose lexicographic order
 * is the strings' order */
int vgk_dict_chunks(const VgStrDict *d, int64_t n_codes, int n_chunks, int64_t *d_out, vg_stream_t s);
int vgk_rank_of(const int32_t *d_perm, int64_t n, int64_t *d_rank, vg_stream_t s);
/* d_out[i] = d_table[d_codes[i]] where row i is valid (else 0) */
int vgk_map_codes(const int64_t *d_table, const int64_t *d_codes, const uint32_t *d_valid, int voff, int64_t n,
                  int64_t *d_out, vg_stream_t s);
/* key word k of the listed group-table slots replaced by d_rank[word] */
int vgk_group_keys_remap(const VgGroupTable *gt, int k, const int32_t *d_slots, int64_t n, const int64_t *d_rank,
                         vg_stream_t s);

/* sort / scan building blocks */
size_t vgk_sort_pairs_scratch(int64_t n);
int vgk_sort_pairs(uint64_t *keys, int32_t *vals, int64_t n, int key_bits, void *scratch,
                   size_t scratch_bytes, vg_stream_t s);
const char *vgk_sort_last_error(void);
/* the stable order of rows 0..n-1 by several keys (arrange) into perm */
size_t vgk_sort_rows_scratch(int64_t n);
int vgk_sort_rows(const VgCol *cols, const int *key_col, const int *desc, int n_keys, int32_t *perm, int64_t n,
                  void *scratch, size_t scratch_bytes, vg_stream_t s);
size_t vgk_scan_scratch(int64_t n);
int vgk_exclusive_scan(const int32_t *in, int64_t n, int64_t *out, int64_t *d_total, void *scratch,
                       size_t scratch_bytes, vg_stream_t s);

/* aggregation extras */
const char *vgk_agg_last_error(void);
size_t vgk_lacc_bytes(int64_t cap);
/* replay shared-cache entries spilled by vgk_agg_launch (n of them) */
int vgk_agg_merge_spilled_cache(const VgAggLaunch *L, int64_t n, vg_stream_t s);
/* move every group of `from` into the empty, larger table `to` */
int vgk_group_table_rehash(const VgGroupTable *from, const VgGroupTable *to, int n_keys,
                           const int32_t *key_types, const int32_t *acc_cls, int n_accs,
                           vg_stream_t s);
/* bytes of spilled cache entries per entry (cache layout, one slot) */
size_t vgk_agg_cache_bytes(const VgAggLaunch *L, int64_t slots);

/* payload copy of a unique-key single-key join table: cols[0..n) of the
 * build rows, (cap + 1) entries; key: the build key column (direct tables
 * are filled in build-row order from it) */
int vgk_join_payload(const VgJoinTable *jt, const VgCol *key, const VgCol *cols, int n_cols, VgJPay *pay,
                     vg_stream_t s);

/* run-time specialised aggregation kernel (jit_agg.cu): launch returns 1
 * if launched, 0 if the plan shape is not covered, -1 on error */
int vgk_agg_launch_jit(const VgAggLaunch *L, int64_t n_logical, vg_stream_t s);
int vgk_agg_jit_ok(const VgAggLaunch *L);
int vgk_agg_jit_slots(const VgAggLaunch *L);
int vgk_agg_jit_compile_only(const VgAggLaunch *L, int *regs_out);
int vgk_agg_jit_source(const VgAggLaunch *L, int S, char *out, size_t out_bytes);
const char *vgk_jit_error(void);
unsigned long long vgk_jit_compiles(void);

/* partitioned aggregation (k_pagg.cu, jit_agg.cu) */
int vgk_pagg_groups(const VgAggLaunch *L);          /* groups per reducer CTA, 0 = does not fit */
/* the same with `ctas` reducer CTAs sharing one SM's shared memory */
int vgk_pagg_groups_for(const VgAggLaunch *L, int ctas);
int vgk_pagg_record_words(const VgAggLaunch *L);
int vgk_pagg_source(const VgAggLaunch *L, const VgFinish *fin, int n_out, int G, char *out, size_t out_bytes);
int vgk_pagg_compile_only(const VgAggLaunch *L, const VgFinish *fin, int n_out, int G, int threads,
                          int *regs_out);
/* ctas: reducer CTAs per SM (1: 1024 threads; 2, 4 or 8: 512, 256 or 128 threads each, G sized for
 * that share of the shared memory) */
int vgk_pagg_reduce(const VgAggLaunch *L, const VgFinish *fin, int n_out, int G, int ctas, const VgPaggReduce *B,
                    vg_stream_t s);
const char *vgk_pagg_last_error(void);
/* distinct-key estimate and the order-word range (min, max, valid count)
 * of an int64 key column; d_regs: 4096 words, d_mm: 3 words */
int vgk_pagg_sketch(const VgCol *key, int64_t n, const int32_t *sel, uint32_t *d_regs, unsigned long long *d_mm,
                    double *h_distinct, uint64_t *h_mm, vg_stream_t s);
int vgk_pagg_hist(const VgCol *key, int64_t n, const int32_t *sel, uint64_t omin, int shift, int nb, uint32_t *d_cnt,
                  vg_stream_t s);
/* off[0..nb]: exclusive scan of d_cnt (or, d_cnt NULL, of the bucket sizes
 * of the regions); d_cursor (optional): d_cursor[b * cursor_stride] = off[b] */
int vgk_pagg_scan(const uint32_t *d_cnt, const VgPaggReduce *regions, int64_t nb, uint64_t *d_off,
                  unsigned long long *d_cursor, int cursor_stride, vg_stream_t s);
int vgk_pagg_cursor_compact(const unsigned long long *padded, int stride, int64_t nb, unsigned long long *dense,
                            vg_stream_t s);
/* launch geometry of the fused kernel for L over n rows: grid and rows per
 * CTA tile (CTA c processes tiles c, c + grid, ...) */
int vgk_agg_jit_geometry(const VgAggLaunch *L, int64_t n, int *grid, int64_t *tile);
/* counts of valid keys per (bucket, CTA) over the fused kernel's tiles:
 * M[b * grid + c]; nb <= VG_PAGG_CTA_BUCKETS */
int vgk_pagg_hist_cta(const VgCol *key, int64_t n, const int32_t *sel, uint64_t omin, int shift, int nb, int grid,
                      int64_t tile, uint32_t *d_m, vg_stream_t s);
/* out[0..n]: exclusive scan of n u32 counts (out[n] = total); d_sums:
 * (n / 16384 + 1) words of scratch */
int vgk_scan_u32_u64(const uint32_t *in, int64_t n, uint64_t *out, unsigned long long *d_sums, vg_stream_t s);
int vgk_pagg_rec_minmax(const VgPaggReduce *R, int b, uint64_t rows, unsigned long long *d_mm, uint64_t *h_mm,
                        vg_stream_t s);
int vgk_pagg_rec_split(const VgPaggReduce *R, int b, uint64_t rows, uint64_t omin, int shift, int nb, uint32_t *d_cnt,
                       uint64_t *d_off, unsigned long long *d_cursor, uint64_t *d_out, uint32_t *d_err,
                       vg_stream_t s);
int vgk_pagg_emit(int64_t n_leaves, const uint64_t *d_leaf_stage, const uint64_t *d_leaf_out, int64_t n_groups,
                  int has_na, uint64_t na_stage, const uint64_t *st_key, const uint32_t *st_ok,
                  const double *const *st_out, int n_out, uint64_t *key_out, uint32_t *key_valid, double **out,
                  uint32_t **out_valid, uint64_t out_base, vg_stream_t s);
/* the results of one group-table slot written to staging position pos */
int vgk_group_stage(const VgGroupTable *gt, const VgFinish *fin, int n_out, int64_t slot, uint64_t *st_key,
                    uint32_t *st_ok, double *const *st_out, uint64_t pos, uint32_t *d_warn, vg_stream_t s);
#endif  /* !__CUDACC_RTC__ */

#ifdef __cplusplus
}
#endif

#endif
