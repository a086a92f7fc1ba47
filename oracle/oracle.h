/*
 * oracle.h - CPU restatement of the reference's algorithms for ComputeQL's GPU operator path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker: the tests, the smoke check and the
 * CPU-baseline leg of the bench call it to compute what the reference computes on the same inputs.
 * The product (computeql_gb300) never links or calls it.
 *
 * Every function cites the reference file:line it follows. Parity of this restatement is pinned
 * against the reference's own known answers: the closed-form expectations of
 * src/tests/scale/bench_select_scale.c:97-160 for the closed-form table of :172-198 (see
 * tests/test_oracle_pins.py), and the exact HyperLogLog / t-digest edge cases of
 * src/tests/bench_query_approx_agg.c:428-478.
 */
#ifndef CQL_ORACLE_H
#define CQL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* CQL_ColumnType (src/cql/cql.h:79-95) */
#define ORC_U32 1
#define ORC_U64 2
#define ORC_F32 3
#define ORC_F64 4
#define ORC_I32 7
#define ORC_I64 8

/* Threads the parallel functions may use (0 = all online cores). */
void orc_set_threads(uint32_t n);
uint32_t orc_threads(void);

/* ---- data ---- */
/* splitmix64 (src/tests/bench_common.h:30-37): draw k (0-based) of the stream seeded `seed`. */
uint64_t orc_splitmix_draw(uint64_t seed, uint64_t k);
/* out[r] = draw(r * per_row + index) % range (range 0 = the low 32 bits). */
void orc_fill_splitmix_u32(uint32_t* out, uint64_t rows, uint64_t seed, uint32_t per_row, uint32_t index, uint64_t range);
/* The closed-form scale table of src/tests/scale/bench_select_scale.c:172-198:
   id = i + 1, region_id = i % 50, amount = i % 10000, needle_key = (U32)(i * 2654435761). */
void orc_fill_closed_form(uint32_t* id, uint32_t* region, uint32_t* amount, uint32_t* needle_key, uint64_t rows);

/* ---- whole-column aggregates ---- */
/* qe_aggregate_global_chunked (src/query_exec/query_exec.c:9114-9230): rows split by tp_divide_work
   (src/thread_pool/thread_pool.c:236-249) into `tasks` ranges per 64M-row chunk, each folded in
   double, folded again in task order. */
void orc_aggregate_global_cpu(const void* values, uint32_t type, uint64_t rows, uint32_t tasks, double* out_sum, double* out_min, double* out_max);
/* The reference GPU kernel's order (aggregate_global_native.comp:168-271 + qe_agg_stream_retire
   query_exec.c:8812-8841): 2048 workgroups x 256 threads, 16-byte vectors a grid apart, a workgroup
   tree fold, then the host fold in workgroup order, per 16M-row chunk. */
void orc_aggregate_global_gpu_order(const void* values, uint32_t type, uint64_t rows, double* out_sum, double* out_min, double* out_max);
/* Neumaier-compensated double sum of a column widened to double: the error reference for f64 sums. */
double orc_compensated_sum(const void* values, uint32_t type, uint64_t rows);

/* ---- scan + filter ---- */
typedef struct OrcLeaf
{
  const void* values;   /* the column */
  uint32_t type;        /* ORC_U32 / ORC_I32 / ORC_F32 / ORC_F64 */
  uint32_t op;          /* 0 ==, 1 <, 2 <=, 3 >, 4 >= */
  double target;
} OrcLeaf;
/* AND of comparisons, each value widened to double and compared with the target as the
   reference's CPU scan does (qe_cpu_scan_filter, query_exec.c:14064-14138; compare_rows in
   scan_simple.comp:214-300). Returns the match count; writes up to `cap` matching rows ascending. */
uint64_t orc_scan_and(const OrcLeaf* leaves, uint32_t leaf_count, uint64_t rows, uint32_t* out_rows, uint64_t cap);

/* The scan bytecode (opcodes of src/query_exec/query_exec.h:58-81) evaluated row by row with a double
   stack, as the reference's interpreter scan_filter.comp:325-559 and its CPU scan compute a WHERE
   clause. slot_data[s] is the column of slot s (a raw string column: bytes at s, u64 offsets at
   s + 1), slot_types[s] its CQL type. Writes out_match[r] = 1 for a matching row; returns the count. */
uint64_t orc_eval_program(const uint32_t* words, uint32_t word_count, const uint32_t* consts, const uint8_t* str_pool,
                          const void* const* slot_data, const uint32_t* slot_types, uint64_t rows, uint8_t* out_match);
/* the same with each row's last fuzzy score (SIMILARITY as its f32 value, EDIT_DISTANCE as an integer) */
uint64_t orc_eval_program_scored(const uint32_t* words, uint32_t word_count, const uint32_t* consts, const uint8_t* str_pool,
                                 const void* const* slot_data, const uint32_t* slot_types, uint64_t rows, uint8_t* out_match, double* out_score);

/* A batch of programs over one table (the batched shared scan's answers): the interpreter above run a block
   of rows at a time over every program, threads over row ranges. slot_data / slot_types: programs x 10;
   sum_data[q]: the column program q sums (NULL: COUNT only) of type sum_types[q]. Writes each program's
   match count and the Neumaier-compensated sum of its summed column over the matching rows; returns 0 if a
   program holds an opcode other than the numeric ones. */
int orc_batch_count_sum(uint32_t programs, const uint32_t* const* words, const uint32_t* word_counts, const uint32_t* const* consts,
                        const void* const* slot_data, const uint32_t* slot_types, const void* const* sum_data, const uint32_t* sum_types,
                        uint64_t rows, uint64_t* out_count, double* out_sum);

/* ---- sketches ---- */
/* HyperLogLog registers of a set of values (hll_add, src/gpu/vulkan/shaders/aggregate_reduce.comp:66-92):
   h = hash_u32(lo ^ hash_u32(hi)) of the value's f64 bits, bucket = top p bits, rho from the leading
   one of the rest; regs[bucket] = max(regs, rho). regs has 2^p entries and is not cleared here. */
void orc_hll_add(const double* values, uint64_t n, uint32_t p, uint32_t* regs);
/* qe_hll_estimate_cardinality (src/query_exec/query_exec.c:6711-6737), not rounded. */
double orc_hll_estimate(const uint32_t* regs, uint64_t m);
/* qe_tdigest_estimate_percentile (src/query_exec/query_exec.c:6748-6790) over (mean, weight) centroids; sorts them. */
double orc_tdigest_percentile(float* means, float* weights, uint64_t count, double fraction);

/* ---- dense GROUP BY ---- */
/* Per group g = key - min_key over [0, groups): the count, and per expression the 64-bit
   two's-complement sum, the min and the max of the argument column (as the reference's dense path
   computes them: qe_dense_stream_core, query_exec.c:7632-7983 with aggregate_dense_native.comp).
   funcs: 0 COUNT, 1 SUM, 2 AVG, 3 MIN, 4 MAX. args[e] points at a U32 or I32 column (arg_types[e]). */
void orc_group_dense(const uint32_t* key, uint32_t key_type, uint64_t rows, int64_t min_key, uint64_t groups, uint32_t expr_count,
                     const uint32_t* funcs, const uint32_t* const* args, const uint32_t* arg_types, uint64_t* out_counts,
                     int64_t* out_sums, int64_t* out_mins, int64_t* out_maxs);
/* The reference's single-threaded CPU GROUP BY (qe_aggregate_cpu_reduce, query_exec.c:7295-7392):
   an open-addressing table in first-appearance order with double accumulators. Writes per group
   (first-appearance order) its key, count and per expression sum/min/max; returns the group count. */
uint64_t orc_group_cpu_reduce(const uint32_t* key, uint64_t rows, uint32_t expr_count, const uint32_t* const* args, uint64_t max_groups,
                              uint32_t* out_keys, uint64_t* out_counts, double* out_sums, double* out_mins, double* out_maxs);

#ifdef __cplusplus
}
#endif


/* ORDER BY over key_count F64 key columns laid out key-major (keys[k * rows + i]); desc[k] != 0 for DESC.
   Writes the row numbers in order, ties by position (query_exec.c:4859-4940). */
int orc_sort_rows(const double* keys, uint32_t key_count, const uint32_t* desc, uint64_t rows, uint64_t* out);
int orc_window_rank(const double* keys, uint32_t key_count, const uint32_t* desc, uint32_t partition_count, uint64_t rows, uint64_t* out_rows,
                    uint32_t* row_number, uint32_t* rank, uint32_t* dense_rank);

/* SELECT group, COUNT(*), SUM(fact_arg) over fact JOIN dim ON fact_key = dim_key, dim_group[d] the
   group of dimension row d (0xffffffff = the row is filtered out); fact_arg may be NULL. */
int orc_join_aggregate(const uint32_t* fact_key, const uint32_t* fact_arg, uint64_t rows, const uint32_t* dim_key,
                       const uint32_t* dim_group, uint64_t dim_count, uint32_t groups, uint64_t* out_counts, int64_t* out_sums);

/* qe_values_fixed_point for one task (query_exec.c:3893-3983): the scale (or -1) and the largest |v|. */
int orc_fixed_scale(const double* values, uint64_t count, int32_t* out_scale, double* out_largest);
/* the smallest scale at which each value alone is whole (-1: none up to 6, or |v| >= 2^31) */
void orc_fixed_scale_each(const double* values, uint64_t count, int8_t* out);
/* the dense fixed-point reduce and finalize (aggregate_dense_f64.comp:73-145, query_exec.c:11011-11060);
   keys as f64 whole numbers; returns the present groups, written in key order */
uint64_t orc_dense_fixed(const double* keys, uint64_t rows, uint32_t expr_count, const uint32_t* funcs, const double* const* args,
                         const int32_t* scales, int64_t min_key, uint64_t groups, int64_t* out_keys, uint64_t* out_first_rows,
                         uint64_t* out_counts, double* out_results);
#endif
