/*
 * cql_ops_hash.c - hash GROUP BY with COUNT/SUM/AVG/MIN/MAX, APPROX_COUNT_DISTINCT (HyperLogLog) and
 * APPROX_PERCENTILE (t-digest), driven through the cqlcuda C ABI the way the reference's
 * qe_aggregate_impl drives its GPU (src/query_exec/query_exec.c:10258-12300):
 *
 *   1. keys and arguments as dense f64 (numeric) or raw bytes + offsets (strings)      :10454-10690
 *   2. aggregate_assign into buckets x K slots, buckets grown on overflow and retried   :10792-11243
 *   3. aggregate_compact: occupied slots to dense group ids                             :11251-11330
 *   4a. whole-number arguments: aggregate_hash_reduce_fixed, per-row atomics            :11611-11790
 *   4b. otherwise: csr_scatter into member lists, aggregate_reduce per 4096-row chunk,
 *       HyperLogLog registers and t-digest centroids, folded on the host in chunk order :11826-12275
 *   5. qe_hll_estimate_cardinality (:6711-6737, rounded :12230) and
 *      qe_tdigest_estimate_percentile (:6748-6790)
 */
#include "cqlops.h"
#include "cql_ops_internal.h"

#include <math.h>
#include <stdio.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#define QE_GPU_WORKGROUP_SIZE 256
#define EMPTY 0xffffffffu
#define AGG_ROWS_PER_CHUNK 4096
/* from this many groups on, a warp's rows rarely share a group: per-row atomics instead of combining
   the warp's lanes of one group first */
#define AGG_MANY_GROUPS 4096
#define HLL_PRECISION 10
#define HLL_SKETCH_MAX_BYTES (64ull << 20)

/* The HyperLogLog registers of the calling thread's last hash GROUP BY, [group][hll expression][2^p] */
static __thread uint32_t* tl_hll_regs = NULL;
static __thread uint64_t tl_hll_words = 0;

uint64_t cqlops_group_hash_registers(uint32_t* out, uint64_t capacity)
{
  if (out && tl_hll_regs) memcpy(out, tl_hll_regs, (capacity < tl_hll_words ? capacity : tl_hll_words) * 4);
  return tl_hll_words;
}

static void keep_hll_registers(uint32_t* regs, uint64_t words)
{
  free(tl_hll_regs);
  tl_hll_regs = regs;
  tl_hll_words = regs ? words : 0;
}

static int refuse(const char* why)
{
  cqlops_note_error(why);
  return 0;
}

static CqlBuffer* pooled(const char* name, uint64_t size, uint32_t flags)
{
  return cqlcuda_buffer_alloc_pooled(name, (uint64_t)strlen(name), size ? size : 4, flags, NULL);
}

static CqlKernel* kernel(const char* name)
{
  return cqlcuda_kernel_alloc(name, (uint64_t)strlen(name));
}

/* qe_hll_estimate_cardinality (query_exec.c:6711-6737) */
double cqlops_hll_estimate(const uint32_t* registers, uint64_t m_count)
{
  double m = (double)m_count;
  double alpha = m_count == 16 ? 0.673 : m_count == 32 ? 0.697 : m_count == 64 ? 0.709 : 0.7213 / (1.0 + 1.079 / m);
  double sum = 0.0;
  uint64_t zeros = 0;
  for (uint64_t i = 0; i < m_count; i++)
  {
    sum += 1.0 / (double)((uint64_t)1 << registers[i]);
    if (registers[i] == 0) zeros++;
  }
  double estimate = alpha * m * m / sum;
  if (estimate <= 2.5 * m && zeros > 0) estimate = m * log(m / (double)zeros);
  return estimate;
}

typedef struct
{
  float mean;
  float weight;
} Centroid;

static int centroid_cmp(const void* a, const void* b)
{
  float x = ((const Centroid*)a)->mean, y = ((const Centroid*)b)->mean;
  return (x > y) - (x < y);
}

/* qe_tdigest_estimate_percentile (query_exec.c:6748-6790) */
double cqlops_tdigest_percentile(float* means, float* weights, uint64_t count, double fraction)
{
  if (count == 0) return 0.0;
  Centroid* c = (Centroid*)malloc(sizeof(Centroid) * count);
  if (!c) return 0.0;
  for (uint64_t i = 0; i < count; i++)
  {
    c[i].mean = means[i];
    c[i].weight = weights[i];
  }
  qsort(c, count, sizeof(Centroid), centroid_cmp);
  double total = 0.0;
  for (uint64_t i = 0; i < count; i++) total += c[i].weight;
  double result;
  if (total <= 0.0) result = 0.0;
  else
  {
    double target = fraction * total, cumulative = 0.0, prev_pos = -1.0, prev_mean = (double)c[0].mean;
    result = (double)c[count - 1].mean;
    for (uint64_t i = 0; i < count; i++)
    {
      double pos = cumulative + (double)c[i].weight * 0.5;
      if (target <= pos)
      {
        if (prev_pos < 0.0) result = (double)c[i].mean;
        else
        {
          double t = (target - prev_pos) / (pos - prev_pos);
          result = prev_mean + t * ((double)c[i].mean - prev_mean);
        }
        break;
      }
      cumulative += c[i].weight;
      prev_pos = pos;
      prev_mean = (double)c[i].mean;
    }
  }
  free(c);
  return result;
}

/* a numeric device column widened to a dense f64 buffer (a full-width f64 column is its own) */
static CqlBuffer* widen(const CqlColumn* col, const char* name)
{
  if (col->width != 0 || !col->buffer) return NULL;
  if (col->type == CQLOPS_TYPE_F64) return col->buffer;
  CqlBuffer* out = pooled(name, col->rows * 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* k = kernel("cql_widen_f64");
  if (!out || !k) return NULL;
  cqlcuda_kernel_set_arg_buffer(k, 0, col->buffer);
  cqlcuda_kernel_set_arg_buffer(k, 1, out);
  cqlcuda_kernel_set_arg_u64(k, 0, col->rows);
  cqlcuda_kernel_set_arg_u64(k, 1, col->type);
  CqlBatch* b = cqlcuda_batch_begin(0, 0);
  cqlcuda_batch_kernel_execute(b, k, (uint32_t)(col->rows < 0xffffffffull ? col->rows : 0xffffffffull), QE_GPU_WORKGROUP_SIZE);
  return cqlcuda_batch_end(b) ? out : NULL;
}

static int whole_number_arg(const CqlColumn* col)
{
  return (col->type == CQLOPS_TYPE_U32 || col->type == CQLOPS_TYPE_I32) && col->has_range && col->zone_min >= -2147483648.0 &&
         col->zone_max <= 2147483647.0;
}

/* The CSR member reduce of the groups found by assign/compact: slot_counts/slot_group (compact
   offsets) per slot, group_counts per group, row_slot per row. Writes out_results[g * exprs + e].
   With row_slot NULL there is one group of every row in order (no key). */
typedef struct
{
  CqlBuffer* buffer;
  void* dst;
  uint64_t bytes;
} PendingRead;

/* `open` (optional): a batch the caller began, which the chunk pass joins and ends after the caller's
   `reads` - one wait for both */
static int csr_reduce(uint64_t rows, uint64_t slots, uint64_t groups, CqlBuffer* slot_counts, CqlBuffer* slot_group,
                      CqlBuffer* group_counts, CqlBuffer* row_slot, uint32_t expr_count, const uint32_t* funcs, uint32_t func_codes,
                      CqlBuffer* const* arg_f64, const double* params, double* out_results, CqlBatch* open, const PendingRead* reads,
                      uint32_t read_count)
{
  uint64_t gb = (groups + 255) / 256;
  CqlBuffer* g_start = pooled("agg_group_start_buf", (groups + 1) * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* g_chunks = pooled("agg_group_chunks_buf", groups * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* c_base = pooled("agg_chunk_base_buf", (groups + 1) * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* scratch = pooled("agg_scan_scratch_buf", groups * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* block_sums = pooled("agg_scan_block_buf", gb * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* kchunks = kernel("cql_group_chunks");
  CqlKernel* scan = kernel("prefix_sum");
  if (!g_start || !g_chunks || !c_base || !scratch || !block_sums || !kchunks || !scan)
  {
    if (open) cqlcuda_batch_end(open);
    return 0;
  }
  uint32_t total_chunks32 = 0;
  {
    CqlBatch* b = open ? open : cqlcuda_batch_begin(0, 4);
    cqlcuda_kernel_set_arg_buffer(kchunks, 0, group_counts);
    cqlcuda_kernel_set_arg_buffer(kchunks, 1, g_chunks);
    cqlcuda_kernel_set_arg_u64(kchunks, 0, groups);
    cqlcuda_kernel_set_arg_u64(kchunks, 1, AGG_ROWS_PER_CHUNK);
    cqlcuda_batch_kernel_execute(b, kchunks, (uint32_t)groups, QE_GPU_WORKGROUP_SIZE);
    for (int pass = 0; pass < 2; pass++)
    {
      cqlcuda_kernel_set_arg_buffer(scan, 0, pass ? g_chunks : group_counts);
      cqlcuda_kernel_set_arg_buffer(scan, 1, pass ? c_base : g_start);
      cqlcuda_kernel_set_arg_buffer(scan, 2, scratch);
      cqlcuda_kernel_set_arg_buffer(scan, 3, block_sums);
      cqlcuda_kernel_set_arg_u64(scan, 0, groups);
      for (uint32_t mode = 0; mode < 3; mode++)
      {
        cqlcuda_kernel_set_arg_u64(scan, 1, mode);
        cqlcuda_batch_kernel_execute(b, scan, mode == 1 ? 256u : (uint32_t)(gb * 256), 256);
      }
    }
    /* the caller's reads, then the chunk count: the scan's total, after the last chunk base */
    for (uint32_t r = 0; r < read_count; r++) cqlcuda_batch_buffer_read(b, reads[r].buffer, reads[r].dst, reads[r].bytes);
    cqlcuda_batch_buffer_read_at(b, c_base, groups * 4, &total_chunks32, 4);
    if (!cqlcuda_batch_end(b)) return 0;
  }
  uint64_t total_chunks = total_chunks32;
  uint32_t num_hll = 0, num_pct = 0, hll_slot_packed = 0, pct_slot_packed = 0;
  for (uint32_t e = 0; e < expr_count; e++)
  {
    if (funcs[e] == CQLOPS_FUNC_APPROX_COUNT_DISTINCT) hll_slot_packed |= (num_hll++) << (4 * e);
    if (funcs[e] == CQLOPS_FUNC_APPROX_PERCENTILE) pct_slot_packed |= (num_pct++) << (4 * e);
  }
  uint64_t hll_words = 1ull << HLL_PRECISION;
  uint64_t sketch_bytes = (groups ? groups : 1) * (num_hll ? num_hll : 1) * hll_words * 4;
  uint64_t digest_words = total_chunks * (num_pct ? num_pct : 1) * 256;
  if (num_hll && sketch_bytes > HLL_SKETCH_MAX_BYTES) return refuse("the HyperLogLog sketches exceed QE_HLL_SKETCH_MAX_TOTAL_BYTES (64 MB)");
  CqlBuffer* cursor_buf = pooled("agg_cursor_buf", slots * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* members = pooled("agg_members_buf", rows * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* range_buf = pooled("agg_chunk_range_buf", total_chunks * 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* group_buf = pooled("agg_chunk_group_buf", total_chunks * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* repr_buf = pooled("agg_repr_buf", groups * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* partials_buf = pooled("agg_partials_buf", total_chunks * expr_count * 32, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* results_buf = pooled("agg_results_buf", groups * expr_count * 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* sketch_buf = pooled("agg_sketch_buf", sketch_bytes, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* dmean_buf = pooled("agg_digest_mean_buf", digest_words * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* dweight_buf = pooled("agg_digest_weight_buf", digest_words * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* kcursor = kernel("cql_slot_cursor");
  CqlKernel* kranges = kernel("cql_chunk_ranges");
  CqlKernel* scatter = kernel("csr_scatter");
  CqlKernel* reduce = kernel("aggregate_reduce");
  CqlKernel* fold = kernel("cql_group_fold");
  uint32_t* sketch = num_hll ? (uint32_t*)malloc(sketch_bytes) : NULL;
  float* dmean = num_pct ? (float*)malloc(digest_words * 4) : NULL;
  float* dweight = num_pct ? (float*)malloc(digest_words * 4) : NULL;
  uint32_t* h_base = num_pct ? (uint32_t*)malloc((groups + 1) * 4) : NULL;
  int ok = cursor_buf && members && range_buf && group_buf && repr_buf && partials_buf && results_buf && sketch_buf && dmean_buf &&
           dweight_buf && kcursor && kranges && scatter && reduce && fold && (!num_hll || sketch) && (!num_pct || (dmean && dweight && h_base));
  if (ok)
  {
    if (!row_slot)
    {
      /* one group of all rows in order: the members are the row numbers */
      ok = cqlcuda_fill_sequence_u32(members, rows, 0);
    }
    cqlcuda_kernel_set_arg_buffer(kcursor, 0, slot_counts ? slot_counts : group_counts);
    cqlcuda_kernel_set_arg_buffer(kcursor, 1, slot_group ? slot_group : group_counts);
    cqlcuda_kernel_set_arg_buffer_range(kcursor, 2, g_start, 0, groups * 4);
    cqlcuda_kernel_set_arg_buffer(kcursor, 3, cursor_buf);
    cqlcuda_kernel_set_arg_u64(kcursor, 0, slots);
    cqlcuda_kernel_set_arg_buffer(kranges, 0, g_start);
    cqlcuda_kernel_set_arg_buffer(kranges, 1, group_counts);
    cqlcuda_kernel_set_arg_buffer(kranges, 2, c_base);
    cqlcuda_kernel_set_arg_buffer(kranges, 3, range_buf);
    cqlcuda_kernel_set_arg_buffer(kranges, 4, group_buf);
    cqlcuda_kernel_set_arg_u64(kranges, 0, groups);
    cqlcuda_kernel_set_arg_u64(kranges, 1, AGG_ROWS_PER_CHUNK);
    cqlcuda_kernel_set_arg_buffer(scatter, 0, row_slot ? row_slot : members);
    cqlcuda_kernel_set_arg_buffer(scatter, 1, cursor_buf);
    cqlcuda_kernel_set_arg_buffer(scatter, 2, members);
    cqlcuda_kernel_set_arg_u64(scatter, 0, rows);
    cqlcuda_kernel_set_arg_u64(scatter, 1, groups >= AGG_MANY_GROUPS);
    cqlcuda_kernel_set_arg_buffer(reduce, 0, members);
    cqlcuda_kernel_set_arg_buffer(reduce, 1, range_buf);
    cqlcuda_kernel_set_arg_buffer(reduce, 2, group_buf);
    cqlcuda_kernel_set_arg_buffer(reduce, 3, repr_buf);
    cqlcuda_kernel_set_arg_buffer(reduce, 4, partials_buf);
    for (uint32_t e = 0; e < 8; e++) cqlcuda_kernel_set_arg_buffer(reduce, 5 + e, arg_f64[e] ? arg_f64[e] : members);
    cqlcuda_kernel_set_arg_buffer(reduce, 13, sketch_buf);
    cqlcuda_kernel_set_arg_buffer(reduce, 14, dmean_buf);
    cqlcuda_kernel_set_arg_buffer(reduce, 15, dweight_buf);
    cqlcuda_kernel_set_arg_u64(reduce, 0, total_chunks);
    cqlcuda_kernel_set_arg_u64(reduce, 1, expr_count);
    cqlcuda_kernel_set_arg_u64(reduce, 2, func_codes);
    cqlcuda_kernel_set_arg_u64(reduce, 3, 0);
    cqlcuda_kernel_set_arg_u64(reduce, 4, HLL_PRECISION);
    cqlcuda_kernel_set_arg_u64(reduce, 5, hll_slot_packed);
    cqlcuda_kernel_set_arg_u64(reduce, 6, num_hll);
    cqlcuda_kernel_set_arg_u64(reduce, 7, num_pct | ((uint64_t)pct_slot_packed << 32));
    cqlcuda_kernel_set_arg_buffer(fold, 0, partials_buf);
    cqlcuda_kernel_set_arg_buffer(fold, 1, c_base);
    cqlcuda_kernel_set_arg_buffer(fold, 2, results_buf);
    cqlcuda_kernel_set_arg_u64(fold, 0, groups);
    cqlcuda_kernel_set_arg_u64(fold, 1, expr_count);
    cqlcuda_kernel_set_arg_u64(fold, 2, func_codes);
    CqlBatch* b = cqlcuda_batch_begin(0, groups * expr_count * 8 + sketch_bytes + 2 * digest_words * 4 + (groups + 1) * 4);
    if (num_hll) cqlcuda_batch_buffer_zero(b, sketch_buf, sketch_bytes);
    if (row_slot) cqlcuda_batch_kernel_execute(b, kcursor, (uint32_t)slots, QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_kernel_execute(b, kranges, (uint32_t)groups, QE_GPU_WORKGROUP_SIZE);
    if (row_slot) cqlcuda_batch_kernel_execute(b, scatter, (uint32_t)rows, QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_kernel_execute(b, reduce, (uint32_t)(total_chunks * QE_GPU_WORKGROUP_SIZE), QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_kernel_execute(b, fold, (uint32_t)groups, QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_buffer_read(b, results_buf, out_results, groups * expr_count * 8);
    if (num_hll) cqlcuda_batch_buffer_read(b, sketch_buf, sketch, sketch_bytes);
    if (num_pct)
    {
      cqlcuda_batch_buffer_read(b, dmean_buf, dmean, digest_words * 4);
      cqlcuda_batch_buffer_read(b, dweight_buf, dweight, digest_words * 4);
      cqlcuda_batch_buffer_read(b, c_base, h_base, (groups + 1) * 4);
    }
    ok = cqlcuda_batch_end(b);
  }
  if (ok && (num_hll || num_pct))
  {
    /* the sketches are finished on the host: qe_hll_estimate_cardinality, rounded (:12230), and the
       t-digest percentile over a group's centroids in chunk order (:6748-6790) */
    float* cm = NULL;
    float* cw = NULL;
    for (uint64_t g = 0; g < groups && ok; g++)
      for (uint32_t e = 0; e < expr_count && ok; e++)
      {
        if (funcs[e] == CQLOPS_FUNC_APPROX_COUNT_DISTINCT)
          out_results[g * expr_count + e] =
            round(cqlops_hll_estimate(&sketch[(g * num_hll + ((hll_slot_packed >> (4 * e)) & 0xfu)) * hll_words], hll_words));
        else if (funcs[e] == CQLOPS_FUNC_APPROX_PERCENTILE)
        {
          uint64_t n = h_base[g + 1] - h_base[g], cap = n * 256, v = 0;
          float* m2 = (float*)realloc(cm, (cap ? cap : 1) * 4);
          float* w2 = (float*)realloc(cw, (cap ? cap : 1) * 4);
          if (m2) cm = m2;
          if (w2) cw = w2;
          if (!m2 || !w2)
          {
            ok = 0;
            break;
          }
          uint32_t ps = (pct_slot_packed >> (4 * e)) & 0xfu;
          for (uint64_t k = 0; k < n; k++)
          {
            uint64_t base = ((h_base[g] + k) * num_pct + ps) * 256;
            for (uint32_t t = 0; t < 256; t++)
              if (dweight[base + t] > 0.0f)
              {
                cm[v] = dmean[base + t];
                cw[v] = dweight[base + t];
                v++;
              }
          }
          out_results[g * expr_count + e] = cqlops_tdigest_percentile(cm, cw, v, params ? params[e] : 0.5);
        }
      }
    free(cm);
    free(cw);
  }
  if (ok && sketch)
  {
    keep_hll_registers(sketch, sketch_bytes / 4);
    sketch = NULL;
  }
  free(sketch);
  free(dmean);
  free(dweight);
  free(h_base);
  return ok;
}

/* ---- path 3: a small-range key with COUNT/SUM/AVG/MIN/MAX of f32/f64 columns, in one pass ----
   A key of at most 64 values: one pass over the key and the argument columns (cql_group_small) gives per
   value its count, first row, exact fixed-point SUMs (so the result does not depend on the order of the
   rows) and MIN/MAX. Gives way (-1) when the query does not fit, and to the fixed-point path when every
   f32/f64 argument is a decimal of at most 6 places (that path finalizes them as the reference does). */
#define SMALL_KEY_VALUES 64

static double order_key_to_double(uint64_t k)
{
  uint64_t b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  double v;
  memcpy(&v, &b, 8);
  return v;
}

static int numeric_full(const CqlColumn* c, uint64_t rows)
{
  return c && c->rows == rows && c->width == 0 && c->buffer &&
         (c->type == CQLOPS_TYPE_U32 || c->type == CQLOPS_TYPE_I32 || c->type == CQLOPS_TYPE_F32 || c->type == CQLOPS_TYPE_F64);
}

/* The one-pass form of the small-key GROUP BY (cql_group_small): the key and up to 8 distinct argument
   columns read once, each SUM exact in fixed point at a binary scale chosen from the column's range (a
   whole-number column at scale 0), MIN and MAX as order keys. 1 done, 0 failed. */
#define GROUP_SMALL_COLUMNS 8
static int group_small_fused(const CqlColumn* key, uint32_t values, int64_t kmin, uint32_t expr_count, const uint32_t* funcs,
                             const CqlColumn* const* args, uint64_t max_groups, uint64_t* out_group_count, uint64_t* out_repr_row,
                             uint64_t* out_counts, double* out_results)
{
  uint64_t rows = key->rows;
  const CqlColumn* cols[GROUP_SMALL_COLUMNS];
  uint32_t ncols = 0, need = 0, types = 0, col_of[8] = { 0 };
  int scale[GROUP_SMALL_COLUMNS] = { 0, 0, 0, 0, 0, 0, 0, 0 };
  for (uint32_t e = 0; e < expr_count; e++)
  {
    uint32_t f = funcs[e];
    if (f == CQLOPS_FUNC_COUNT) continue;
    const CqlColumn* c = args[e];
    uint32_t i = 0;
    while (i < ncols && cols[i]->buffer != c->buffer) i++;
    if (i == ncols)
    {
      cols[ncols++] = c;
      types |= (c->type & 0xfu) << (4 * i);
    }
    col_of[e] = i;
    need |= (f == CQLOPS_FUNC_SUM || f == CQLOPS_FUNC_AVG) ? (1u << i) : (1u << (GROUP_SMALL_COLUMNS + i));
  }
  /* each summed f32/f64 column's largest finite magnitude: from its zone range, or (no range, or an infinite
     one) from one pass over it */
  double largest[GROUP_SMALL_COLUMNS] = { 0 };
  uint64_t measured[GROUP_SMALL_COLUMNS] = { 0 };
  uint32_t measure_mask = 0;
  for (uint32_t i = 0; i < ncols; i++)
  {
    const CqlColumn* c = cols[i];
    if (!((need >> i) & 1u) || c->type == CQLOPS_TYPE_U32 || c->type == CQLOPS_TYPE_I32) continue;
    if (c->has_range && isfinite(c->zone_min) && isfinite(c->zone_max))
      largest[i] = fabs(c->zone_min) > fabs(c->zone_max) ? fabs(c->zone_min) : fabs(c->zone_max);
    else
      measure_mask |= 1u << i;
  }
  if (measure_mask)
  {
    CqlBuffer* mb = pooled("group_small_magnitude", GROUP_SMALL_COLUMNS * 8, CQLCUDA_BUFFER_READ_WRITE);
    CqlKernel* mk = kernel("cql_finite_magnitude");
    if (!mb || !mk) return 0;
    CqlBatch* b = cqlcuda_batch_begin(0, GROUP_SMALL_COLUMNS * 8);
    cqlcuda_batch_buffer_zero(b, mb, GROUP_SMALL_COLUMNS * 8);
    for (uint32_t i = 0; i < ncols; i++)
    {
      if (!((measure_mask >> i) & 1u)) continue;
      cqlcuda_kernel_set_arg_buffer(mk, 0, cols[i]->buffer);
      cqlcuda_kernel_set_arg_buffer_range(mk, 1, mb, (uint64_t)i * 8, 8);
      cqlcuda_kernel_set_arg_u64(mk, 0, rows);
      cqlcuda_kernel_set_arg_u64(mk, 1, cols[i]->type);
      cqlcuda_batch_kernel_execute(b, mk, (uint32_t)rows, QE_GPU_WORKGROUP_SIZE);
    }
    cqlcuda_batch_buffer_read(b, mb, measured, GROUP_SMALL_COLUMNS * 8);
    if (!cqlcuda_batch_end(b)) return 0;
    for (uint32_t i = 0; i < ncols; i++)
      if ((measure_mask >> i) & 1u) memcpy(&largest[i], &measured[i], 8);
  }
  for (uint32_t i = 0; i < ncols; i++)
  {
    const CqlColumn* c = cols[i];
    if (!((need >> i) & 1u) || c->type == CQLOPS_TYPE_U32 || c->type == CQLOPS_TYPE_I32) continue;   /* scale 0: exact */
    int e2 = 0;
    if (largest[i] > 0.0) frexp(largest[i], &e2);   /* largest < 2^e2 */
    int sc = 61 - e2;                                /* |x| * 2^sc < 2^61 */
    scale[i] = sc > 1023 ? 1023 : sc < -1022 ? -1022 : sc;
  }
  uint64_t words = 3ull * values + (values & 1u) + 9ull * GROUP_SMALL_COLUMNS * values;
  uint32_t sums_at = 3u * values + (values & 1u);
  CqlBuffer* ob = pooled("group_small_out", words * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* k = kernel("cql_group_small");
  uint32_t* host = (uint32_t*)calloc(words, 4);
  if (!ob || !k || !host)
  {
    free(host);
    return 0;
  }
  for (uint32_t v = 0; v < values; v++) host[2 * values + v] = 0xffffffffu;
  uint64_t* ext = (uint64_t*)(host + sums_at + 5u * GROUP_SMALL_COLUMNS * values);
  for (uint32_t i = 0; i < values * GROUP_SMALL_COLUMNS; i++) ext[2 * i] = ~0ull;
  uint64_t packed_scales[2] = { 0, 0 };
  for (uint32_t i = 0; i < GROUP_SMALL_COLUMNS; i++) packed_scales[i / 4] |= (uint64_t)(uint16_t)(int16_t)scale[i] << (16 * (i % 4));
  cqlcuda_kernel_set_arg_buffer(k, 0, key->buffer);
  for (uint32_t i = 0; i < GROUP_SMALL_COLUMNS; i++) cqlcuda_kernel_set_arg_buffer(k, 1 + i, i < ncols ? cols[i]->buffer : key->buffer);
  cqlcuda_kernel_set_arg_buffer(k, 1 + GROUP_SMALL_COLUMNS, ob);
  cqlcuda_kernel_set_arg_u64(k, 0, rows);
  cqlcuda_kernel_set_arg_u64(k, 1, (uint32_t)kmin);
  cqlcuda_kernel_set_arg_u64(k, 2, values);
  cqlcuda_kernel_set_arg_u64(k, 3, ncols);
  cqlcuda_kernel_set_arg_u64(k, 4, types);
  cqlcuda_kernel_set_arg_u64(k, 5, need);
  cqlcuda_kernel_set_arg_u64(k, 6, packed_scales[0]);
  cqlcuda_kernel_set_arg_u64(k, 7, packed_scales[1]);
  CqlBatch* b = cqlcuda_batch_begin(words * 4, words * 4);
  cqlcuda_batch_buffer_write(b, ob, host, words * 4);
  cqlcuda_batch_kernel_execute(b, k, (uint32_t)rows, QE_GPU_WORKGROUP_SIZE);
  cqlcuda_batch_buffer_read(b, ob, host, words * 4);
  int result = cqlcuda_batch_end(b) ? 1 : 0;
  const uint64_t* counts = (const uint64_t*)host;
  const uint32_t* first = host + 2 * values;
  const uint64_t* sums = (const uint64_t*)(host + sums_at);
  const uint32_t* flags = host + sums_at + 4u * GROUP_SMALL_COLUMNS * values;
  uint64_t g = 0;
  for (uint32_t v = 0; v < values && result == 1; v++)
  {
    uint64_t count = counts[v];
    if (count == 0) continue;
    if (g >= max_groups)
    {
      result = refuse("more groups than the output arrays hold");
      break;
    }
    out_repr_row[g] = first[v];
    out_counts[g] = count;
    for (uint32_t e = 0; e < expr_count; e++)
    {
      uint32_t f = funcs[e], i = col_of[e], at = v * GROUP_SMALL_COLUMNS + i;
      double r = (double)count;
      if (f == CQLOPS_FUNC_SUM || f == CQLOPS_FUNC_AVG)
      {
        /* the 128-bit total, rounded once to a double and scaled back by 2^-s; NaN and infinities as IEEE sums give them */
        __int128 total = (__int128)(((unsigned __int128)sums[2 * at + 1] << 64) | sums[2 * at]);
        uint32_t fl = flags[at];
        double sum = ldexp((double)total, -scale[i]);
        if ((fl & 1u) || (fl & 6u) == 6u) sum = NAN;
        else if (fl & 2u) sum = INFINITY;
        else if (fl & 4u) sum = -INFINITY;
        r = f == CQLOPS_FUNC_AVG ? sum / (double)count : sum;
      }
      else if (f == CQLOPS_FUNC_MIN || f == CQLOPS_FUNC_MAX)
      {
        /* a group whose values are all NaN keeps the member reduce's starting values */
        uint64_t o = ext[2 * at + (f == CQLOPS_FUNC_MAX)];
        int empty = f == CQLOPS_FUNC_MIN ? o == ~0ull : o == 0ull;
        r = empty ? (f == CQLOPS_FUNC_MIN ? 1.0e300 : -1.0e300) : order_key_to_double(o);
      }
      out_results[g * expr_count + e] = r;
    }
    g++;
  }
  if (result == 1) *out_group_count = g;
  free(host);
  return result;
}

static int group_small_key(const CqlColumn* key, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* args, uint64_t max_groups,
                           uint64_t* out_group_count, uint64_t* out_repr_row, uint64_t* out_counts, double* out_results)
{
  if (!(key->type == CQLOPS_TYPE_U32 || key->type == CQLOPS_TYPE_I32) || key->width != 0 || !key->buffer || !key->has_range) return -1;
  double span = key->zone_max - key->zone_min;
  if (!(span >= 0.0) || span + 1.0 > (double)SMALL_KEY_VALUES) return -1;
  uint32_t values = (uint32_t)span + 1u;
  int64_t kmin = (int64_t)key->zone_min;
  uint64_t rows = key->rows;
  uint32_t fractional = 0;
  for (uint32_t e = 0; e < expr_count; e++)
  {
    uint32_t f = funcs[e];
    if (f == CQLOPS_FUNC_COUNT) continue;
    const CqlColumn* c = args[e];
    if (f > CQLOPS_FUNC_MAX || !numeric_full(c, rows)) return -1;
    if (c->type == CQLOPS_TYPE_F32 || c->type == CQLOPS_TYPE_F64) fractional = 1;
  }
  if (!fractional) return -1;   /* whole numbers: the fixed-point hash reduce is exact already */
  /* decimals of at most 6 places take the fixed-point reduce, which finalizes them as the reference does */
  int all_decimal = 1;
  for (uint32_t e = 0; e < expr_count && all_decimal; e++)
  {
    const CqlColumn* c = args[e];
    if (funcs[e] == CQLOPS_FUNC_COUNT || (c->type != CQLOPS_TYPE_F32 && c->type != CQLOPS_TYPE_F64)) continue;
    int32_t scale = -1;
    double largest = 0.0;
    if (!cqlops_fixed_scale(c, NULL, rows, &scale, &largest) || scale < 0) all_decimal = 0;
  }
  cqlops_note_error("");
  if (all_decimal) return -1;
  return group_small_fused(key, values, kmin, expr_count, funcs, args, max_groups, out_group_count, out_repr_row, out_counts, out_results);
}

/* ---- path 4: one whole-number key of a dense range too large for shared memory, in tables indexed by key ----
   A key whose zone range holds 65537 to 2^24 values (past the dense group-by's 65536 and at most 8 times the
   rows) with whole-number COUNT/SUM/AVG/MIN/MAX: counts, first rows, sums (i64), minimums and maximums (i32)
   in device tables indexed by key - min (cql_group_direct: a few MB, which stay in L2), then the present keys
   listed in key order and the groups written in the caller's layout on the device. No hashing, no member
   pass; the results are those of the fixed-point reduce at scale 0. Gives way (-1) when the query does not
   fit. */
#define DIRECT_MIN_VALUES 65537ull
#define DIRECT_MAX_VALUES (1ull << 24)

static int group_direct(const CqlColumn* key, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* args, uint64_t max_groups,
                        uint64_t* out_group_count, uint64_t* out_repr_row, uint64_t* out_counts, double* out_results)
{
  if (!(key->type == CQLOPS_TYPE_U32 || key->type == CQLOPS_TYPE_I32) || key->width != 0 || !key->buffer || !key->has_range) return -1;
  double span = key->zone_max - key->zone_min;
  uint64_t rows = key->rows;
  if (!(span >= 0.0) || span + 1.0 > (double)DIRECT_MAX_VALUES || span + 1.0 < (double)DIRECT_MIN_VALUES || span + 1.0 > 8.0 * (double)rows)
    return -1;
  uint32_t R = (uint32_t)span + 1u;
  uint32_t func_codes = 0, signed_args = 0, offsets[8] = { 0 };
  uint64_t words = 2ull * R;
  for (uint32_t e = 0; e < expr_count; e++)
  {
    uint32_t f = funcs[e];
    if (f > CQLOPS_FUNC_MAX) return -1;
    func_codes |= f << (4 * e);
    if (f == CQLOPS_FUNC_COUNT) continue;
    const CqlColumn* c = args[e];
    if (!c || c->rows != rows || c->width != 0 || !c->buffer || !whole_number_arg(c)) return -1;
    if (c->type == CQLOPS_TYPE_I32) signed_args |= 1u << e;
    if (f == CQLOPS_FUNC_SUM || f == CQLOPS_FUNC_AVG)
    {
      words = (words + 1) & ~1ull;   /* i64 tables start 8-byte aligned */
      offsets[e] = (uint32_t)words;
      words += 2ull * R;
    }
    else
    {
      offsets[e] = (uint32_t)words;
      words += R;
    }
  }
  if (words > 0xffffffffull) return -1;
  uint64_t most = R < rows ? R : rows;
  uint64_t out_cap = most < max_groups ? most : max_groups;
  if (out_cap == 0) out_cap = 1;
  CqlBuffer* tab = pooled("group_direct_tables", words * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* bits = pooled("group_direct_bits", ((R + 31ull) / 32) * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* present = pooled("group_direct_present", 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* list = pooled("group_direct_list", most * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* repr = pooled("group_direct_repr", out_cap * 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* cnts = pooled("group_direct_counts", out_cap * 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* res = pooled("group_direct_results", out_cap * 8 * expr_count, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* k = kernel("cql_group_direct");
  CqlKernel* kb = kernel("cql_group_direct_bits");
  CqlKernel* ke = kernel("cql_group_direct_emit");
  if (!tab || !bits || !present || !list || !repr || !cnts || !res || !k || !kb || !ke) return 0;
  cqlcuda_kernel_set_arg_buffer(k, 0, key->buffer);
  for (uint32_t e = 0; e < 8; e++)
    cqlcuda_kernel_set_arg_buffer(k, 1 + e, e < expr_count && funcs[e] != CQLOPS_FUNC_COUNT ? args[e]->buffer : key->buffer);
  cqlcuda_kernel_set_arg_buffer(k, 9, tab);
  cqlcuda_kernel_set_arg_u64(k, 0, rows);
  cqlcuda_kernel_set_arg_u64(k, 1, (uint64_t)(uint32_t)(int64_t)key->zone_min | ((uint64_t)R << 32));
  cqlcuda_kernel_set_arg_u64(k, 2, (uint64_t)expr_count | ((uint64_t)func_codes << 32));
  cqlcuda_kernel_set_arg_u64(k, 3, signed_args);
  for (uint32_t i = 0; i < 4; i++) cqlcuda_kernel_set_arg_u64(k, 4 + i, (uint64_t)offsets[2 * i] | ((uint64_t)offsets[2 * i + 1] << 32));
  cqlcuda_kernel_set_arg_buffer(kb, 0, tab);
  cqlcuda_kernel_set_arg_buffer(kb, 1, bits);
  cqlcuda_kernel_set_arg_buffer(kb, 2, present);
  cqlcuda_kernel_set_arg_u64(kb, 0, R);
  cqlcuda_kernel_set_arg_buffer(ke, 0, tab);
  cqlcuda_kernel_set_arg_buffer(ke, 1, list);
  cqlcuda_kernel_set_arg_buffer(ke, 2, present);
  cqlcuda_kernel_set_arg_buffer(ke, 3, repr);
  cqlcuda_kernel_set_arg_buffer(ke, 4, cnts);
  cqlcuda_kernel_set_arg_buffer(ke, 5, res);
  for (uint32_t i = 0; i < 8; i++) cqlcuda_kernel_set_arg_u64(ke, i, 0);
  cqlcuda_kernel_set_arg_u64(ke, 1, (uint64_t)R << 32);
  cqlcuda_kernel_set_arg_u64(ke, 2, (uint64_t)expr_count | ((uint64_t)func_codes << 32));
  for (uint32_t i = 0; i < 4; i++) cqlcuda_kernel_set_arg_u64(ke, 4 + i, (uint64_t)offsets[2 * i] | ((uint64_t)offsets[2 * i + 1] << 32));
  uint32_t groups = 0;
  CqlBatch* b = cqlcuda_batch_begin(0, 4);
  cqlcuda_batch_fill_range(b, tab, 0, (uint64_t)R * 4, 0);
  cqlcuda_batch_fill_range(b, tab, (uint64_t)R * 4, (uint64_t)R * 4, 0xffffffffu);
  for (uint32_t e = 0; e < expr_count; e++)
  {
    uint32_t f = funcs[e];
    if (f == CQLOPS_FUNC_COUNT) continue;
    uint64_t at = (uint64_t)offsets[e] * 4;
    if (f == CQLOPS_FUNC_SUM || f == CQLOPS_FUNC_AVG) cqlcuda_batch_fill_range(b, tab, at, (uint64_t)R * 8, 0);
    else cqlcuda_batch_fill_range(b, tab, at, (uint64_t)R * 4, f == CQLOPS_FUNC_MIN ? 0x7fffffffu : 0x80000000u);
  }
  cqlcuda_batch_buffer_zero(b, present, 4);
  cqlcuda_batch_kernel_execute(b, k, (uint32_t)rows, QE_GPU_WORKGROUP_SIZE);
  cqlcuda_batch_kernel_execute(b, kb, R, QE_GPU_WORKGROUP_SIZE);
  if (!cqlops_bitmap_rows_enqueue(b, bits, 0, R, list))
  {
    cqlcuda_batch_end(b);
    return 0;
  }
  cqlcuda_batch_kernel_execute(b, ke, (uint32_t)most, QE_GPU_WORKGROUP_SIZE);
  cqlcuda_batch_buffer_read(b, present, &groups, 4);
  if (!cqlcuda_batch_end(b)) return 0;
  if (groups > max_groups) return refuse("more groups than the output arrays hold");
  if (groups)
  {
    b = cqlcuda_batch_begin(0, (uint64_t)groups * (16 + 8ull * expr_count));
    cqlcuda_batch_buffer_read(b, repr, out_repr_row, (uint64_t)groups * 8);
    cqlcuda_batch_buffer_read(b, cnts, out_counts, (uint64_t)groups * 8);
    cqlcuda_batch_buffer_read(b, res, out_results, (uint64_t)groups * 8 * expr_count);
    if (!cqlcuda_batch_end(b)) return 0;
  }
  *out_group_count = groups;
  return 1;
}

int cqlops_group_hash(const CqlColumn* keys, uint32_t key_count, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* args,
                      const double* params, uint64_t group_hint, uint32_t path, uint64_t max_groups, uint64_t* out_group_count,
                      uint64_t* out_repr_row, uint64_t* out_counts, double* out_results, uint32_t* out_path)
{
  cqlops_note_error("");
  keep_hll_registers(NULL, 0);
  if (key_count > 4 || expr_count == 0 || expr_count > 8) return refuse("0 to 4 keys and 1 to 8 aggregates");
  /* no GROUP BY: one bucket of one slot takes every row (:10796-10801) */
  uint64_t rows = key_count ? keys[0].rows : 0;
  for (uint32_t e = 0; e < expr_count && !key_count; e++)
    if (args[e]) rows = args[e]->rows;
  if (!cqlops_rows_fit(rows)) return 0;
  if (rows == 0)
  {
    /* no rows, no groups: an aggregate over nothing is the caller's empty result */
    *out_group_count = 0;
    if (out_path) *out_path = 0;
    return 1;
  }
  if ((path == 0 || path == 3) && key_count == 1)
  {
    int r = group_small_key(&keys[0], expr_count, funcs, args, max_groups, out_group_count, out_repr_row, out_counts, out_results);
    if (r >= 0)
    {
      if (r == 1 && out_path) *out_path = 3;
      return r;
    }
    if (path == 3) return refuse("path 3 takes one whole-number key of at most 64 values with COUNT/SUM/AVG/MIN/MAX over f32/f64 columns");
    cqlops_note_error("");
  }
  if ((path == 0 || path == 4) && key_count == 1)
  {
    int r = group_direct(&keys[0], expr_count, funcs, args, max_groups, out_group_count, out_repr_row, out_counts, out_results);
    if (r >= 0)
    {
      if (r == 1 && out_path) *out_path = 4;
      return r;
    }
    if (path == 4)
      return refuse("path 4 takes one whole-number key of 65537 to 2^24 values (at most 8 per row) with whole-number COUNT/SUM/AVG/MIN/MAX");
    cqlops_note_error("");
  }
  uint32_t key_types = 0;   /* per key: its CQL type when bound at its stored width, 0 = widened to f64 */
  uint32_t string_mask = 0;
  CqlBuffer* key_data[4] = { 0 };
  CqlBuffer* key_off[4] = { 0 };
  char name[64];
  for (uint32_t c = 0; c < key_count; c++)
  {
    if (keys[c].rows != rows) return refuse("keys of different lengths");
    if (keys[c].type == CQLOPS_TYPE_STRING8)
    {
      if (!keys[c].offsets || keys[c].dict) return refuse("a string key is read as raw bytes and offsets");
      string_mask |= 1u << c;
      key_data[c] = keys[c].buffer;
      key_off[c] = keys[c].offsets;
    }
    else if (keys[c].width == 0 && keys[c].buffer &&
             (keys[c].type == CQLOPS_TYPE_U32 || keys[c].type == CQLOPS_TYPE_I32 || keys[c].type == CQLOPS_TYPE_F32))
    {
      /* read at its stored width and widened to f64 in the assign kernel's registers */
      key_data[c] = keys[c].buffer;
      key_off[c] = keys[c].buffer;
      key_types |= keys[c].type << (4 * c);
    }
    else
    {
      snprintf(name, sizeof(name), "cqlops_hash_key_f64_%u", c);
      key_data[c] = widen(&keys[c], name);
      if (!key_data[c]) return refuse("a key column could not be widened to f64 (narrow or sequence encodings are not taken here)");
      key_off[c] = key_data[c];
    }
  }
  int has_sketch = 0, all_whole = 1;
  uint32_t fixed_scales = 0;
  uint32_t func_codes = 0;
  for (uint32_t e = 0; e < expr_count; e++)
  {
    if (funcs[e] > CQLOPS_FUNC_APPROX_PERCENTILE) return refuse("unsupported aggregate function");
    func_codes |= (funcs[e] & 0xfu) << (4 * e);
    if (funcs[e] == CQLOPS_FUNC_APPROX_COUNT_DISTINCT || funcs[e] == CQLOPS_FUNC_APPROX_PERCENTILE) has_sketch = 1;
    if (funcs[e] != CQLOPS_FUNC_COUNT)
    {
      if (!args[e] || args[e]->rows != rows) return refuse("an aggregate needs an argument column of the table's length");
      if (whole_number_arg(args[e]))
        continue;
      /* an f64 argument of decimals with at most 6 places reduces as scaled integers too (:10896-10913) */
      int32_t scale = -1;
      double largest = 0.0;
      if (args[e]->type == CQLOPS_TYPE_F64 && funcs[e] <= CQLOPS_FUNC_MAX && args[e]->width == 0 &&
          !cqlops_fixed_scale(args[e], NULL, 0, &scale, &largest))
        return 0;
      cqlops_note_error("");
      if (scale < 0) all_whole = 0;
      else fixed_scales |= (uint32_t)scale << (4 * e);
    }
  }
  int use_fixed = !has_sketch && all_whole && key_count > 0;
  if (path == 1) use_fixed = 0;
  if (path == 2 && (!use_fixed)) return refuse("the fixed-point reduce takes whole-number COUNT/SUM/AVG/MIN/MAX only");
  CqlBuffer* arg_f64[8] = { 0 };
  for (uint32_t e = 0; e < expr_count; e++)
  {
    if (funcs[e] == CQLOPS_FUNC_COUNT) continue;
    snprintf(name, sizeof(name), "cqlops_hash_arg_f64_%u", e);
    arg_f64[e] = widen(args[e], name);
    if (!arg_f64[e]) return refuse("an argument column could not be widened to f64");
  }

  if (key_count == 0)
  {
    /* no key: one group of every row, its members the rows in order - no hash table, no scatter */
    CqlBuffer* one = pooled("agg_single_group_count_buf", 4, CQLCUDA_BUFFER_READ_WRITE);
    if (!one || max_groups < 1) return one ? refuse("more groups than the output arrays hold") : 0;
    uint32_t n32 = (uint32_t)rows;
    CqlBatch* b = cqlcuda_batch_begin(4, 0);
    cqlcuda_batch_buffer_write(b, one, &n32, 4);
    if (!cqlcuda_batch_end(b)) return 0;
    out_repr_row[0] = 0;
    out_counts[0] = rows;
    if (!csr_reduce(rows, 1, 1, NULL, NULL, one, NULL, expr_count, funcs, func_codes, arg_f64, params, out_results, NULL, NULL, 0)) return 0;
    *out_group_count = 1;
    if (out_path) *out_path = 1u;
    return 1;
  }

  /* buckets: ~64 rows per group unless the caller knows better (:10792-10826) */
  uint64_t max_buckets = 1;
  while (max_buckets < rows) max_buckets <<= 1;
  uint64_t buckets = 16;
  if (key_count == 0)
  {
    buckets = 1;
    max_buckets = 1;
  }
  else if (group_hint > 0)
  {
    uint64_t wanted = group_hint + group_hint / 4;
    while (buckets < wanted && buckets < max_buckets) buckets <<= 1;
  }
  else
    while (buckets < rows / 64 && buckets < max_buckets) buckets <<= 1;
  uint64_t K = key_count ? 8 : 1;
  /* GB300 layout: with keys, linear probing over a power-of-two table of about twice the expected groups
     (K = the probe limit), which for a million groups stays in L2; the reference's buckets of K slots
     (buckets 1.25 x the groups) would be 16 slots a group, larger than L2 and read whole by compaction */
  int linear = key_count > 0;
  if (linear)
  {
    uint64_t want = group_hint > 0 ? 2 * group_hint : rows / 32;
    max_buckets = 1024;
    while (max_buckets < 2 * rows) max_buckets <<= 1;
    buckets = 1024;
    while (buckets < want && buckets < max_buckets) buckets <<= 1;
    K = 64;
  }
  CqlKernel* assign = kernel("aggregate_assign");
  CqlKernel* compact = kernel("aggregate_compact");
  if (!assign || !compact) return 0;
  CqlBuffer *owner = NULL, *count = NULL, *row_slot = NULL, *overflow = NULL;
  CqlBuffer *offsets = NULL, *out_owner = NULL, *out_count = NULL;
  uint64_t slots = 0;
  uint32_t groups32 = 0;
  for (int attempt = 0; attempt < 16; attempt++)
  {
    slots = linear ? buckets : buckets * K;
    owner = pooled("agg_owner_buf", slots * 4, CQLCUDA_BUFFER_READ_WRITE);
    count = pooled("agg_count_buf", slots * 4, CQLCUDA_BUFFER_READ_WRITE);
    row_slot = pooled("agg_row_slot_buf", rows * 4, CQLCUDA_BUFFER_READ_WRITE);
    overflow = pooled("agg_overflow_buf", 4, CQLCUDA_BUFFER_READ_WRITE);
    /* compaction: offsets[slot] becomes the dense group id of an occupied slot */
    uint64_t blocks = (slots + 255) / 256;
    uint64_t max_g = slots < rows ? slots : rows;
    offsets = pooled("agg_compact_offsets_buf", (slots + 1) * 4, CQLCUDA_BUFFER_READ_WRITE);
    CqlBuffer* block_sums = pooled("agg_compact_block_sum_buf", blocks * 4, CQLCUDA_BUFFER_READ_WRITE);
    out_owner = pooled("agg_compact_owner_buf", max_g * 4, CQLCUDA_BUFFER_READ_WRITE);
    out_count = pooled("agg_compact_count_buf", max_g * 4, CQLCUDA_BUFFER_READ_WRITE);
    CqlBuffer* total_buf = pooled("agg_compact_total_buf", 4, CQLCUDA_BUFFER_READ_WRITE);
    if (!owner || !count || !row_slot || !overflow || !offsets || !block_sums || !out_owner || !out_count || !total_buf) return 0;
    for (uint32_t c = 0; c < 4; c++)
    {
      /* key bindings past the key count are never read: bound to the row-slot buffer */
      cqlcuda_kernel_set_arg_buffer(assign, 4 + 2 * c, c < key_count ? key_data[c] : row_slot);
      cqlcuda_kernel_set_arg_buffer(assign, 5 + 2 * c, c < key_count ? key_off[c] : row_slot);
    }
    cqlcuda_kernel_set_arg_buffer(assign, 0, owner);
    cqlcuda_kernel_set_arg_buffer(assign, 1, count);
    cqlcuda_kernel_set_arg_buffer(assign, 2, row_slot);
    cqlcuda_kernel_set_arg_buffer(assign, 3, overflow);
    cqlcuda_kernel_set_arg_u64(assign, 0, rows);
    cqlcuda_kernel_set_arg_u64(assign, 1, buckets);
    cqlcuda_kernel_set_arg_u64(assign, 2, K);
    cqlcuda_kernel_set_arg_u64(assign, 3, key_count);
    cqlcuda_kernel_set_arg_u64(assign, 4, string_mask);
    cqlcuda_kernel_set_arg_u64(assign, 5, group_hint >= AGG_MANY_GROUPS);
    cqlcuda_kernel_set_arg_u64(assign, 6, linear);
    cqlcuda_kernel_set_arg_u64(assign, 7, key_types);
    cqlcuda_kernel_set_arg_buffer(compact, 0, count);
    cqlcuda_kernel_set_arg_buffer(compact, 1, owner);
    cqlcuda_kernel_set_arg_buffer(compact, 2, offsets);
    cqlcuda_kernel_set_arg_buffer(compact, 3, block_sums);
    cqlcuda_kernel_set_arg_buffer(compact, 4, out_owner);
    cqlcuda_kernel_set_arg_buffer(compact, 5, out_count);
    cqlcuda_kernel_set_arg_buffer(compact, 6, total_buf);
    cqlcuda_kernel_set_arg_u64(compact, 0, slots);
    /* the assignment and its compaction in one batch, one wait: an overflowing table (rare) is compacted for
       nothing and assigned again with more room */
    uint32_t over = 0;
    CqlBatch* b = cqlcuda_batch_begin(0, 8);
    cqlcuda_batch_buffer_fill(b, owner, slots * 4, EMPTY);
    cqlcuda_batch_buffer_zero(b, count, slots * 4);
    cqlcuda_batch_buffer_fill(b, row_slot, rows * 4, EMPTY);
    cqlcuda_batch_buffer_zero(b, overflow, 4);
    cqlcuda_batch_kernel_execute(b, assign, (uint32_t)rows, QE_GPU_WORKGROUP_SIZE);
    cqlcuda_kernel_set_arg_u64(compact, 1, 0);
    cqlcuda_batch_kernel_execute(b, compact, (uint32_t)(blocks * 256), 256);
    cqlcuda_kernel_set_arg_u64(compact, 1, 1);
    cqlcuda_batch_kernel_execute(b, compact, 256, 256);
    cqlcuda_kernel_set_arg_u64(compact, 1, 2);
    cqlcuda_batch_kernel_execute(b, compact, (uint32_t)(blocks * 256), 256);
    cqlcuda_batch_buffer_read(b, overflow, &over, 4);
    cqlcuda_batch_buffer_read(b, total_buf, &groups32, 4);
    if (!cqlcuda_batch_end(b)) return 0;
    if (over == 0 || key_count == 0) break;
    /* grow the buckets by how badly they missed, then K (:11226-11243) */
    if (buckets < max_buckets)
    {
      double frac = (double)over / (double)rows;
      uint64_t growth = frac >= 0.20 ? 8 : (frac >= 0.05 ? 4 : 2);
      buckets = buckets * growth < max_buckets ? buckets * growth : max_buckets;
    }
    else K *= 2;
    if (attempt == 15) return refuse("the group-by hash table kept overflowing");
  }
  uint64_t groups = groups32;
  if (groups > max_groups) return refuse("more groups than the output arrays hold");
  /* the representative rows and counts (and, on the fixed path, the finished results) are written in the
     caller's layout by cql_group_finish and read straight into the caller's arrays */
  CqlBuffer* repr64 = pooled("agg_finish_repr_buf", groups * 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* count64 = pooled("agg_finish_count_buf", groups * 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* finish = kernel("cql_group_finish");
  if (!repr64 || !count64 || !finish) return 0;
  cqlcuda_kernel_set_arg_buffer(finish, 0, out_owner);
  cqlcuda_kernel_set_arg_buffer(finish, 1, out_count);
  cqlcuda_kernel_set_arg_buffer(finish, 2, repr64);
  cqlcuda_kernel_set_arg_buffer(finish, 3, count64);
  for (uint32_t i = 4; i < 8; i++) cqlcuda_kernel_set_arg_buffer(finish, i, out_owner);
  cqlcuda_kernel_set_arg_u64(finish, 0, groups);
  cqlcuda_kernel_set_arg_u64(finish, 1, expr_count);
  cqlcuda_kernel_set_arg_u64(finish, 2, func_codes);
  cqlcuda_kernel_set_arg_u64(finish, 3, fixed_scales);
  cqlcuda_kernel_set_arg_u64(finish, 4, 0);
  int ok = 1;
  if (use_fixed)
  {
    /* 4a: per-row atomics into per-group arrays; the compact offsets are the slot -> group map. A query
       of COUNTs alone needs no reduce: the compacted counts are its results. */
    int reduce = 0, has_min_max = 0;
    for (uint32_t e = 0; e < expr_count; e++)
    {
      if (funcs[e] != CQLOPS_FUNC_COUNT) reduce = 1;
      if (funcs[e] == CQLOPS_FUNC_MIN || funcs[e] == CQLOPS_FUNC_MAX) has_min_max = 1;
    }
    CqlKernel* hr = kernel("aggregate_hash_reduce_fixed");
    uint64_t cells = groups * expr_count;
    CqlBuffer* sums = pooled("agg_hash_sum_buf", cells * 8, CQLCUDA_BUFFER_READ_WRITE);
    CqlBuffer* cnts = pooled("agg_hash_count_buf", cells * 4, CQLCUDA_BUFFER_READ_WRITE);
    CqlBuffer* mins = pooled("agg_hash_min_buf", cells * 4, CQLCUDA_BUFFER_READ_WRITE);
    CqlBuffer* maxs = pooled("agg_hash_max_buf", cells * 4, CQLCUDA_BUFFER_READ_WRITE);
    CqlBuffer* results = pooled("agg_finish_results_buf", cells * 8, CQLCUDA_BUFFER_READ_WRITE);
    ok = hr && sums && cnts && mins && maxs && results;
    if (ok)
    {
      cqlcuda_kernel_set_arg_buffer(hr, 0, row_slot);
      cqlcuda_kernel_set_arg_buffer(hr, 1, offsets);
      cqlcuda_kernel_set_arg_buffer(hr, 2, sums);
      cqlcuda_kernel_set_arg_buffer(hr, 3, cnts);
      cqlcuda_kernel_set_arg_buffer(hr, 4, mins);
      cqlcuda_kernel_set_arg_buffer(hr, 5, maxs);
      for (uint32_t e = 0; e < 8; e++) cqlcuda_kernel_set_arg_buffer(hr, 6 + e, arg_f64[e] ? arg_f64[e] : row_slot);
      cqlcuda_kernel_set_arg_u64(hr, 0, rows);
      cqlcuda_kernel_set_arg_u64(hr, 1, expr_count);
      cqlcuda_kernel_set_arg_u64(hr, 2, func_codes);
      cqlcuda_kernel_set_arg_u64(hr, 3, fixed_scales);
      cqlcuda_kernel_set_arg_u64(hr, 4, groups >= AGG_MANY_GROUPS);
      cqlcuda_kernel_set_arg_buffer(finish, 4, sums);
      cqlcuda_kernel_set_arg_buffer(finish, 5, mins);
      cqlcuda_kernel_set_arg_buffer(finish, 6, maxs);
      cqlcuda_kernel_set_arg_buffer(finish, 7, results);
      cqlcuda_kernel_set_arg_u64(finish, 4, 1);
      CqlBatch* b = cqlcuda_batch_begin(0, groups * 16 + cells * 8);
      if (reduce)
      {
        cqlcuda_batch_buffer_zero(b, sums, cells * 8);
        cqlcuda_batch_buffer_zero(b, cnts, cells * 4);
        if (has_min_max)
        {
          cqlcuda_batch_buffer_fill(b, mins, cells * 4, 0x7fffffffu);
          cqlcuda_batch_buffer_fill(b, maxs, cells * 4, 0x80000000u);
        }
        cqlcuda_batch_kernel_execute(b, hr, (uint32_t)rows, QE_GPU_WORKGROUP_SIZE);
      }
      cqlcuda_batch_kernel_execute(b, finish, (uint32_t)groups, QE_GPU_WORKGROUP_SIZE);
      cqlcuda_batch_buffer_read(b, repr64, out_repr_row, groups * 8);
      cqlcuda_batch_buffer_read(b, count64, out_counts, groups * 8);
      cqlcuda_batch_buffer_read(b, results, out_results, cells * 8);
      ok = cqlcuda_batch_end(b);
    }
  }
  else
  {
    /* 4b: member lists, group g's members at [start[g], start[g] + count[g]), laid out on the device:
       group starts and chunk bases by prefix sums, cursors and chunk ranges by kernels, the member
       reduce per 4096-row chunk, and each group's chunks folded in chunk order (:11826-12215). The
       representative rows and counts are finished in the batch of the chunk pass. */
    CqlBatch* b = cqlcuda_batch_begin(0, groups * 16 + 16);
    cqlcuda_batch_kernel_execute(b, finish, (uint32_t)groups, QE_GPU_WORKGROUP_SIZE);
    PendingRead reads[2] = { { repr64, out_repr_row, groups * 8 }, { count64, out_counts, groups * 8 } };
    ok = csr_reduce(rows, slots, groups, count, offsets, out_count, row_slot, expr_count, funcs, func_codes, arg_f64, params,
                    out_results, b, reads, 2);
  }
  if (ok)
  {
    *out_group_count = groups;
    if (out_path) *out_path = use_fixed ? 2u : 1u;
  }
  return ok;
}
