/*
 * Prints the size and field offsets of every struct of the node contract.
 * Compiled twice (oracle/Makefile `abi`): once against the reference's own
 * headers (src/types.h, expr.h, group_agg.h, join.h, filter.h, project.h)
 * and once against include/vectra_abi.h.  tests/test_abi_layout.py requires
 * identical output; tests/golden/abi_layout.txt holds the reference's copy
 * so the check also runs where the reference checkout is absent.
 * TEST INFRASTRUCTURE ONLY.
 */
#include <stdio.h>
#include <stddef.h>

#ifdef USE_REF_HEADERS
#include "types.h"
#include "expr.h"
#include "agg_ops.h"
#include "group_agg.h"
#include "join.h"
#include "filter.h"
#include "project.h"
#include "vtr1.h"
#include "scan.h"
#include "sort.h"
typedef JoinNode JoinPrefixT;
#else
#include "vectra_abi.h"
typedef JoinNodePrefix JoinPrefixT;
#endif

#define S(T) printf("sizeof %s %zu\n", #T, sizeof(T))
#define O(T, f) printf("offsetof %s.%s %zu\n", #T, #f, offsetof(T, f))

int main(void) {
    S(VecArray); O(VecArray, type); O(VecArray, length); O(VecArray, validity);
    O(VecArray, owns_data); O(VecArray, buf.i64); O(VecArray, buf.str.offsets);
    O(VecArray, buf.str.data); O(VecArray, buf.str.data_len);
    S(VecBatch); O(VecBatch, n_rows); O(VecBatch, n_cols); O(VecBatch, col_names);
    O(VecBatch, columns); O(VecBatch, sel); O(VecBatch, sel_n);
    S(VecSchema); O(VecSchema, n_cols); O(VecSchema, col_names);
    O(VecSchema, col_types); O(VecSchema, col_annotations);
    S(VecNode); O(VecNode, next_batch); O(VecNode, free_node);
    O(VecNode, output_schema); O(VecNode, kind);
    S(VecExpr); O(VecExpr, kind); O(VecExpr, result_type); O(VecExpr, col_name);
    O(VecExpr, lit_i64); O(VecExpr, lit_dbl); O(VecExpr, lit_bln);
    O(VecExpr, lit_str); O(VecExpr, op); O(VecExpr, op2); O(VecExpr, left);
    O(VecExpr, right); O(VecExpr, operand); O(VecExpr, cond);
    O(VecExpr, then_expr); O(VecExpr, else_expr); O(VecExpr, cast_to);
    S(AggSpec); O(AggSpec, output_name); O(AggSpec, kind); O(AggSpec, input_col);
    O(AggSpec, na_rm);
    S(GroupAggNode); O(GroupAggNode, child); O(GroupAggNode, n_keys);
    O(GroupAggNode, key_names); O(GroupAggNode, n_aggs);
    O(GroupAggNode, agg_specs); O(GroupAggNode, done); O(GroupAggNode, use_sorted);
    S(JoinKey); O(JoinKey, left_col); O(JoinKey, right_col);
    O(JoinPrefixT, left); O(JoinPrefixT, right); O(JoinPrefixT, kind);
    O(JoinPrefixT, n_keys); O(JoinPrefixT, keys); O(JoinPrefixT, suffix_x);
    O(JoinPrefixT, suffix_y);
    S(FilterNode); O(FilterNode, child); O(FilterNode, predicate);
    S(ProjEntry); O(ProjEntry, output_name); O(ProjEntry, expr);
    S(ProjectNode); O(ProjectNode, child); O(ProjectNode, n_entries);
    O(ProjectNode, entries);
    S(Vtr1Header); O(Vtr1Header, version); O(Vtr1Header, schema); O(Vtr1Header, n_rowgroups);
    S(Vtr1ColStat); O(Vtr1ColStat, has_stats); O(Vtr1ColStat, i64.min); O(Vtr1ColStat, i64.max);
    O(Vtr1ColStat, dbl.min); O(Vtr1ColStat, dbl.max); O(Vtr1ColStat, bln.min); O(Vtr1ColStat, bln.max);
    S(Vtr1RowGroup); O(Vtr1RowGroup, file_offset); O(Vtr1RowGroup, n_rows); O(Vtr1RowGroup, col_stats);
    S(Vtr1File); O(Vtr1File, fp); O(Vtr1File, header); O(Vtr1File, rowgroups);
    S(ScanNode); O(ScanNode, file); O(ScanNode, col_mask); O(ScanNode, next_rg);
    O(ScanNode, predicate); O(ScanNode, pred_borrowed);
    S(SortKey); O(SortKey, col_index); O(SortKey, descending);
    S(SortNode); O(SortNode, child); O(SortNode, n_keys); O(SortNode, keys); O(SortNode, phase);
    O(SortNode, mem_budget); O(SortNode, temp_dir); O(SortNode, n_runs); O(SortNode, runs_cap);
    O(SortNode, run_paths); O(SortNode, mem_result); O(SortNode, merge);
    printf("enum VEC_STRING %d EXPR_GREPL %d AGG_MAX %d JOIN_ANTI %d\n",
           (int)VEC_STRING, (int)EXPR_GREPL, (int)AGG_MAX, (int)JOIN_ANTI);
    return 0;
}
