/*
 * oracle_fixed.c - decimals as scaled integers, as the reference computes them (TEST INFRASTRUCTURE ONLY).
 *
 * orc_fixed_scale restates qe_fixed_point_task and qe_values_fixed_point
 * (src/query_exec/query_exec.c:3893-3983) for one task: the running scale only goes up, a value
 * whose magnitude is not below 2^31 or that needs more than 6 places fails the column, and the
 * largest magnitude times 10^scale must stay below 2^31. orc_dense_fixed restates the dense
 * fixed-point reduce (src/gpu/vulkan/shaders/aggregate_dense_f64.comp:73-145: q = int(floor(v*10^s + 0.5)),
 * exact 64-bit sums, i32 min/max, the smallest row per group) and its finalize (query_exec.c:11011-11060).
 * All in FP64 exactly as written there (the library is built without contracting a*b+c).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>

#define QE_FIXED_MAX_SCALE 6
#define QE_AGG_FIXED_SCALED_LIMIT 2147483648.0

static const double g_pow10[QE_FIXED_MAX_SCALE + 1] = { 1.0, 10.0, 100.0, 1000.0, 10000.0, 100000.0, 1000000.0 };

static int whole_at(double v, int scale)
{
  double scaled = v * g_pow10[scale];
  double whole = (double)(int64_t)(scaled < 0.0 ? scaled - 0.5 : scaled + 0.5);
  return whole / g_pow10[scale] == v;
}

int orc_fixed_scale(const double* values, uint64_t count, int32_t* out_scale, double* out_largest)
{
  int scale = 0;
  double largest = 0.0;
  for (uint64_t i = 0; i < count; i++)
  {
    double v = values[i];
    double magnitude = v < 0.0 ? -v : v;
    if (!(magnitude < QE_AGG_FIXED_SCALED_LIMIT))
    {
      scale = -1;
      break;
    }
    largest = largest > magnitude ? largest : magnitude;
    for (;;)
    {
      if (whole_at(v, scale)) break;
      scale += 1;
      if (scale > QE_FIXED_MAX_SCALE) break;
    }
    if (scale > QE_FIXED_MAX_SCALE)
    {
      scale = -1;
      break;
    }
  }
  if (scale >= 0 && largest * g_pow10[scale] >= QE_AGG_FIXED_SCALED_LIMIT) scale = -1;
  *out_scale = scale;
  *out_largest = largest;
  return scale >= 0;
}

void orc_fixed_scale_each(const double* values, uint64_t count, int8_t* out)
{
  for (uint64_t i = 0; i < count; i++)
  {
    double v = values[i];
    double magnitude = v < 0.0 ? -v : v;
    int s = 0;
    if (!(magnitude < QE_AGG_FIXED_SCALED_LIMIT))
    {
      out[i] = -1;
      continue;
    }
    while (s <= QE_FIXED_MAX_SCALE && !whole_at(v, s)) s++;
    out[i] = s > QE_FIXED_MAX_SCALE ? (int8_t)-1 : (int8_t)s;
  }
}

uint64_t orc_dense_fixed(const double* keys, uint64_t rows, uint32_t expr_count, const uint32_t* funcs, const double* const* args,
                         const int32_t* scales, int64_t min_key, uint64_t groups, int64_t* out_keys, uint64_t* out_first_rows,
                         uint64_t* out_counts, double* out_results)
{
  uint64_t* count = (uint64_t*)calloc(groups, 8);
  uint64_t* first = (uint64_t*)malloc(groups * 8);
  int64_t* sum = (int64_t*)calloc(groups * expr_count, 8);
  int32_t* mn = (int32_t*)malloc(groups * expr_count * 4);
  int32_t* mx = (int32_t*)malloc(groups * expr_count * 4);
  for (uint64_t i = 0; i < groups; i++) first[i] = UINT64_MAX;
  for (uint64_t i = 0; i < groups * expr_count; i++)
  {
    mn[i] = INT32_MAX;
    mx[i] = INT32_MIN;
  }
  for (uint64_t r = 0; r < rows; r++)
  {
    int64_t id = (int64_t)(int32_t)keys[r] - min_key;
    if (id < 0 || (uint64_t)id >= groups) continue;
    if (r < first[id]) first[id] = r;
    count[id]++;
    for (uint32_t e = 0; e < expr_count; e++)
    {
      if (funcs[e] == 0) continue;
      int32_t q = (int32_t)floor(args[e][r] * g_pow10[scales[e]] + 0.5);
      uint64_t index = (uint64_t)id * expr_count + e;
      if (funcs[e] == 1 || funcs[e] == 2) sum[index] += q;
      else if (funcs[e] == 3) { if (q < mn[index]) mn[index] = q; }
      else if (funcs[e] == 4) { if (q > mx[index]) mx[index] = q; }
    }
  }
  uint64_t out = 0;
  for (uint64_t g = 0; g < groups; g++)
  {
    if (!count[g]) continue;
    out_keys[out] = min_key + (int64_t)g;
    out_first_rows[out] = first[g];
    out_counts[out] = count[g];
    for (uint32_t e = 0; e < expr_count; e++)
    {
      uint64_t index = g * expr_count + e;
      double divisor = g_pow10[scales[e]];
      double value = 0.0;
      switch (funcs[e])
      {
        case 0: value = (double)count[g]; break;
        case 1: value = (double)sum[index] / divisor; break;
        case 2: value = (double)sum[index] / divisor / (double)count[g]; break;
        case 3: value = (double)mn[index] / divisor; break;
        case 4: value = (double)mx[index] / divisor; break;
      }
      out_results[out * expr_count + e] = value;
    }
    out++;
  }
  free(count);
  free(first);
  free(sum);
  free(mn);
  free(mx);
  return out;
}
