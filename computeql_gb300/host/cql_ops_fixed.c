/*
 * cql_ops_fixed.c - decimals aggregated as scaled integers.
 *
 *   cqlops_fixed_scale        qe_values_fixed_point (src/query_exec/query_exec.c:3893-3983) on a device column
 *   cqlops_group_dense_fixed  the dense branch of qe_aggregate_impl (query_exec.c:10917-11083) with its
 *                             fixed-point arguments (:10896-10913): key range, argument scales, one
 *                             reduce, the host finalize of each group's values
 *
 * The reference gathers the key and the arguments to f64 on the host, checks the scales there and
 * uploads both; here the key and the arguments stay in their device columns (u32/i32/f64 key,
 * f64/f32 arguments) and the key range and the scales come from two small reduction kernels.
 */
#include "cqlops.h"
#include "cql_ops_internal.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define QE_GPU_WORKGROUP_SIZE 256
#define QE_FIXED_MAX_SCALE 6
#define QE_AGG_FIXED_SCALED_LIMIT 2147483648.0
#define DENSE_FIXED_MAX_WORDS 51200u

static const double g_pow10[QE_FIXED_MAX_SCALE + 1] = { 1.0, 10.0, 100.0, 1000.0, 10000.0, 100000.0, 1000000.0 };

static int refuse(const char* why)
{
  cqlops_note_error(why);
  return 0;
}

static CqlBuffer* pooled(const char* name, uint64_t size, uint32_t flags)
{
  return cqlcuda_buffer_alloc_pooled(name, (uint64_t)strlen(name), size ? size : 8, flags, NULL);
}

static CqlKernel* kernel(const char* name)
{
  return cqlcuda_kernel_alloc(name, (uint64_t)strlen(name));
}

/* smallest and largest key over the rows (or the selection); 0 when a key is not a whole number in i32 */
static int key_range(const CqlColumn* key, CqlBuffer* selection, uint64_t n, int64_t* out_min, int64_t* out_max)
{
  CqlBuffer* res = pooled("fixed_key_range", 24, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* k = kernel("cql_key_range");
  if (!res || !k) return 0;
  int64_t init[3] = { INT64_MAX, INT64_MIN, 0 };
  int64_t out[3] = { 0, 0, 0 };
  cqlcuda_kernel_set_arg_buffer(k, 0, key->buffer);
  cqlcuda_kernel_set_arg_buffer(k, 1, res);
  cqlcuda_kernel_set_arg_buffer(k, 2, selection ? selection : res);
  cqlcuda_kernel_set_arg_u64(k, 0, n);
  cqlcuda_kernel_set_arg_u64(k, 1, key->type);
  cqlcuda_kernel_set_arg_u64(k, 2, selection ? 1 : 0);
  CqlBatch* b = cqlcuda_batch_begin(24, 24);
  cqlcuda_batch_buffer_write(b, res, init, 24);
  cqlcuda_batch_kernel_execute(b, k, (uint32_t)(n < 0xffffffffull ? n : 0xffffffffull), QE_GPU_WORKGROUP_SIZE);
  cqlcuda_batch_buffer_read(b, res, out, 24);
  if (!cqlcuda_batch_end(b)) return 0;
  if (out[2] & 0xffffffff) return refuse("a key is not a whole number inside the 32-bit range");
  *out_min = out[0];
  *out_max = out[1];
  return 1;
}

int cqlops_fixed_scale(const CqlColumn* column, CqlBuffer* selection, uint64_t selection_count, int32_t* out_scale, double* out_largest)
{
  cqlops_note_error("");
  *out_scale = -1;
  *out_largest = 0.0;
  if (!column || !column->buffer || column->width != 0) return refuse("a full-width numeric column");
  uint64_t n = selection ? selection_count : column->rows;
  if (!cqlops_rows_fit(column->rows) || !cqlops_rows_fit(n)) return 0;
  if (selection && cqlcuda_buffer_size(selection) < n * 4) return refuse("selection buffer smaller than its count");
  if (n == 0)
  {
    *out_scale = 0;
    return 1;
  }
  if (column->type == CQLOPS_TYPE_U32 || column->type == CQLOPS_TYPE_I32)
  {
    /* whole numbers: scale 0 while every magnitude is below 2^31 */
    int64_t lo, hi;
    if (!key_range(column, selection, n, &lo, &hi)) return 0;
    double largest = (double)(hi > -lo ? hi : -lo);
    *out_largest = largest;
    *out_scale = largest < QE_AGG_FIXED_SCALED_LIMIT ? 0 : -1;
    return 1;
  }
  if (column->type != CQLOPS_TYPE_F64 && column->type != CQLOPS_TYPE_F32) return refuse("fixed-point scales are found for numeric columns");
  CqlBuffer* res = pooled("fixed_scale_result", 16, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* k = kernel("cql_fixed_scale");
  if (!res || !k) return 0;
  uint32_t out[4] = { 0, 0, 0, 0 };
  cqlcuda_kernel_set_arg_buffer(k, 0, column->buffer);
  cqlcuda_kernel_set_arg_buffer(k, 1, res);
  cqlcuda_kernel_set_arg_buffer(k, 2, selection ? selection : res);
  cqlcuda_kernel_set_arg_buffer(k, 3, res);
  cqlcuda_kernel_set_arg_u64(k, 0, n);
  cqlcuda_kernel_set_arg_u64(k, 1, column->type);
  cqlcuda_kernel_set_arg_u64(k, 2, selection ? 1 : 0);
  cqlcuda_kernel_set_arg_u64(k, 3, 0);
  CqlBatch* b = cqlcuda_batch_begin(0, 16);
  cqlcuda_batch_buffer_zero(b, res, 16);
  cqlcuda_batch_kernel_execute(b, k, (uint32_t)(n < 0xffffffffull ? n : 0xffffffffull), QE_GPU_WORKGROUP_SIZE);
  cqlcuda_batch_buffer_read(b, res, out, 16);
  if (!cqlcuda_batch_end(b)) return 0;
  uint64_t bits = ((uint64_t)out[3] << 32) | out[2];
  double largest;
  memcpy(&largest, &bits, 8);
  int32_t scale = out[1] ? -1 : (int32_t)out[0];
  /* a larger scale than a range needed makes its values larger, so the whole scaled range is checked (:3975-3979) */
  if (scale >= 0 && largest * g_pow10[scale] >= QE_AGG_FIXED_SCALED_LIMIT) scale = -1;
  *out_scale = scale;
  *out_largest = largest;
  return 1;
}

int cqlops_group_dense_fixed(const CqlColumn* key, uint32_t expr_count, const uint32_t* funcs, const CqlColumn* const* args,
                             CqlBuffer* selection, uint64_t selection_count, uint64_t max_groups, uint64_t* out_groups,
                             int64_t* out_keys, uint64_t* out_first_rows, uint64_t* out_counts, double* out_results, int32_t* out_scales)
{
  cqlops_note_error("");
  *out_groups = 0;
  if (!key || !key->buffer || key->width != 0 ||
      !(key->type == CQLOPS_TYPE_U32 || key->type == CQLOPS_TYPE_I32 || key->type == CQLOPS_TYPE_F64))
    return refuse("dense fixed-point group-by: a full-width U32/I32/F64 key");
  if (expr_count == 0 || expr_count > 8) return refuse("1 to 8 aggregates");
  uint64_t rows = key->rows;
  uint64_t n = selection ? selection_count : rows;
  if (!cqlops_rows_fit(rows)) return 0;
  if (selection && cqlcuda_buffer_size(selection) < n * 4) return refuse("selection buffer smaller than its count");
  uint32_t func_codes = 0, scales = 0, arg_f32 = 0;
  int32_t scale_of[8];
  for (uint32_t e = 0; e < expr_count; e++)
  {
    if (funcs[e] > CQLOPS_FUNC_MAX) return refuse("COUNT/SUM/AVG/MIN/MAX only");
    func_codes |= (funcs[e] & 0xfu) << (4 * e);
    scale_of[e] = 0;
    if (funcs[e] == CQLOPS_FUNC_COUNT) continue;
    const CqlColumn* a = args[e];
    if (!a || a->rows != rows || !a->buffer || a->width != 0 || !(a->type == CQLOPS_TYPE_F64 || a->type == CQLOPS_TYPE_F32))
      return refuse("fixed-point arguments are full-width F64/F32 columns of the key's length");
    if (a->type == CQLOPS_TYPE_F32) arg_f32 |= 1u << e;
    /* one scale per distinct argument column (arg_owner, :10896-10913) */
    uint32_t owner = e;
    for (uint32_t o = 0; o < e; o++)
      if (funcs[o] != CQLOPS_FUNC_COUNT && args[o]->buffer == a->buffer) owner = o;
    if (owner != e)
      scale_of[e] = scale_of[owner];
    else
    {
      double largest;
      if (!cqlops_fixed_scale(a, selection, n, &scale_of[e], &largest)) return 0;
      if (scale_of[e] < 0) return refuse("an argument is not a decimal of at most 6 places below 2^31 once scaled");
    }
    scales |= (uint32_t)scale_of[e] << (4 * e);
  }
  if (out_scales)
    for (uint32_t e = 0; e < expr_count; e++) out_scales[e] = scale_of[e];
  if (n == 0) return 1;
  int64_t kmin, kmax;
  if (!key_range(key, selection, n, &kmin, &kmax)) return 0;
  if (kmin < INT32_MIN || kmax > INT32_MAX) return refuse("key outside the 32-bit range");
  uint64_t groups = (uint64_t)(kmax - kmin) + 1;
  if (groups * (2 + 4 * (uint64_t)expr_count) > DENSE_FIXED_MAX_WORDS) return refuse("the key range is too wide for the dense path");
  if (groups > max_groups) return refuse("more groups than the output holds");
  uint64_t entries = groups * expr_count;
  CqlBuffer* info = pooled("agg_dense_info_buf", groups * 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* sums = pooled("agg_dense_sum_buf", entries * 8, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* mins = pooled("agg_dense_min_buf", entries * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* maxs = pooled("agg_dense_max_buf", entries * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlKernel* k = kernel("cql_dense_fixed");
  uint32_t* info_h = (uint32_t*)malloc(groups * 8);
  int64_t* sum_h = (int64_t*)malloc(entries * 8);
  int32_t* min_h = (int32_t*)malloc(entries * 4);
  int32_t* max_h = (int32_t*)malloc(entries * 4);
  int ok = info && sums && mins && maxs && k && info_h && sum_h && min_h && max_h;
  if (ok)
  {
    cqlcuda_kernel_set_arg_buffer(k, 0, key->buffer);
    cqlcuda_kernel_set_arg_buffer(k, 1, info);
    cqlcuda_kernel_set_arg_buffer(k, 2, sums);
    cqlcuda_kernel_set_arg_buffer(k, 3, mins);
    cqlcuda_kernel_set_arg_buffer(k, 4, maxs);
    for (uint32_t e = 0; e < 8; e++)
      cqlcuda_kernel_set_arg_buffer(k, 5 + e, e < expr_count && funcs[e] != CQLOPS_FUNC_COUNT ? args[e]->buffer : info);
    cqlcuda_kernel_set_arg_buffer(k, 13, selection ? selection : info);
    cqlcuda_kernel_set_arg_u64(k, 0, n);
    cqlcuda_kernel_set_arg_u64(k, 1, expr_count);
    cqlcuda_kernel_set_arg_u64(k, 2, func_codes);
    cqlcuda_kernel_set_arg_u64(k, 3, scales);
    cqlcuda_kernel_set_arg_u64(k, 4, groups);
    cqlcuda_kernel_set_arg_u64(k, 5, (uint64_t)(uint32_t)(int32_t)kmin);
    cqlcuda_kernel_set_arg_u64(k, 6, (uint64_t)key->type | ((uint64_t)arg_f32 << 32));
    cqlcuda_kernel_set_arg_u64(k, 7, selection ? 1 : 0);
    CqlBatch* b = cqlcuda_batch_begin(0, groups * 8 + entries * 16);
    cqlcuda_batch_buffer_zero(b, info, groups * 8);
    cqlcuda_batch_buffer_zero(b, sums, entries * 8);
    cqlcuda_batch_buffer_fill(b, mins, entries * 4, 0x7fffffffu);
    cqlcuda_batch_buffer_fill(b, maxs, entries * 4, 0x80000000u);
    cqlcuda_batch_kernel_execute(b, k, (uint32_t)n, QE_GPU_WORKGROUP_SIZE);
    cqlcuda_batch_buffer_read(b, info, info_h, groups * 8);
    cqlcuda_batch_buffer_read(b, sums, sum_h, entries * 8);
    cqlcuda_batch_buffer_read(b, mins, min_h, entries * 4);
    cqlcuda_batch_buffer_read(b, maxs, max_h, entries * 4);
    ok = cqlcuda_batch_end(b);
  }
  if (ok)
  {
    /* the finalize of each present group, in key order (query_exec.c:11011-11060) */
    uint64_t out = 0;
    for (uint64_t g = 0; g < groups; g++)
    {
      uint32_t count = info_h[g * 2 + 1];
      if (count == 0) continue;
      out_keys[out] = kmin + (int64_t)g;
      out_first_rows[out] = ~info_h[g * 2];
      out_counts[out] = count;
      for (uint32_t e = 0; e < expr_count; e++)
      {
        uint64_t index = g * expr_count + e;
        double divisor = g_pow10[scale_of[e]];
        double value = 0.0;
        switch (funcs[e])
        {
          case CQLOPS_FUNC_COUNT: value = (double)count; break;
          case CQLOPS_FUNC_SUM: value = (double)sum_h[index] / divisor; break;
          case CQLOPS_FUNC_AVG: value = (double)sum_h[index] / divisor / (double)count; break;
          case CQLOPS_FUNC_MIN: value = (double)min_h[index] / divisor; break;
          case CQLOPS_FUNC_MAX: value = (double)max_h[index] / divisor; break;
          default: break;
        }
        out_results[out * expr_count + e] = value;
      }
      out++;
    }
    *out_groups = out;
  }
  free(info_h);
  free(sum_h);
  free(min_h);
  free(max_h);
  return ok;
}
