/*
 * cql_zonemap.c - zone maps and the scan pruning that uses them.
 *
 *   cqlops_zone_map_build  per-chunk min/max of a device column (cql_column_ensure_zone_map), by the
 *                          cql_zone_map kernel
 *   cqlops_scan_ranges     qe_scan_build_dispatch_ranges (src/query_exec/query_exec.c:13307-13540) for a
 *                          table held in one buffer (rows_per_chunk = the whole table)
 *
 * A sequence column (width 3, value = base + row) has an implied zone map: chunk z holds the values of
 * rows z*8192 .. z*8192+8191, so `id = k` keeps the one chunk holding row k.
 */
#include "cqlops.h"
#include "cql_ops_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define QE_GPU_WORKGROUP_SIZE 256
#define ZONEMAP_LOG2 13
#define QE_SCAN_MIN_PRUNE_GAP_ROWS 1048576ull
#define QE_SCAN_MIN_PRUNE_PERCENT 10ull
#define QE_SCAN_RANGE_COST_ROWS 4194304ull

static int refuse(const char* why)
{
  cqlops_note_error(why);
  return 0;
}

/* after the chunks: the largest chunk min and the smallest chunk max (over chunks with values), which
   tell at once whether a leaf can prune any chunk */
static void zone_summary(double* zm, uint64_t chunks)
{
  double max_min = -HUGE_VAL, min_max = HUGE_VAL;
  for (uint64_t z = 0; z < chunks; z++)
  {
    double mn = zm[2 * z], mx = zm[2 * z + 1];
    if (mn > mx) continue;
    if (mn > max_min) max_min = mn;
    if (mx < min_max) min_max = mx;
  }
  zm[2 * chunks] = max_min;
  zm[2 * chunks + 1] = min_max;
}

int cqlops_zone_map_build(const CqlColumn* column, double* out_zone_map, uint64_t out_chunks)
{
  cqlops_note_error("");
  uint64_t rows = column->rows;
  if (!cqlops_rows_fit(rows)) return 0;
  uint64_t chunks = (rows + CQLOPS_ZONEMAP_CHUNK_ROWS - 1) / CQLOPS_ZONEMAP_CHUNK_ROWS;
  if (out_chunks < chunks + 1) return refuse("the zone map needs one entry per chunk and one for the summary");
  if (rows == 0) return 1;
  uint32_t t = column->type;
  if (!(t == CQLOPS_TYPE_U32 || t == CQLOPS_TYPE_I32 || t == CQLOPS_TYPE_F32 || t == CQLOPS_TYPE_F64))
    return refuse("zone maps are kept for numeric columns");
  if (column->width == 3)
  {
    /* a sequence: the map is implied */
    for (uint64_t z = 0; z < chunks; z++)
    {
      uint64_t first = z * CQLOPS_ZONEMAP_CHUNK_ROWS;
      uint64_t last = first + CQLOPS_ZONEMAP_CHUNK_ROWS - 1 < rows - 1 ? first + CQLOPS_ZONEMAP_CHUNK_ROWS - 1 : rows - 1;
      uint32_t a = column->base + (uint32_t)first, b = column->base + (uint32_t)last;
      out_zone_map[2 * z] = t == CQLOPS_TYPE_I32 ? (double)(int32_t)a : (double)a;
      out_zone_map[2 * z + 1] = t == CQLOPS_TYPE_I32 ? (double)(int32_t)b : (double)b;
      if (out_zone_map[2 * z] > out_zone_map[2 * z + 1])
      {
        /* the values wrap inside the chunk: no usable range */
        out_zone_map[2 * z] = -1.0e300;
        out_zone_map[2 * z + 1] = 1.0e300;
      }
    }
    zone_summary(out_zone_map, chunks);
    return 1;
  }
  if (!column->buffer || column->width > 2) return refuse("a stored column");
  const char* name = "cql_zone_map_out";
  CqlBuffer* out = cqlcuda_buffer_alloc_pooled(name, strlen(name), chunks * 16, CQLCUDA_BUFFER_READ_WRITE, NULL);
  CqlKernel* k = cqlcuda_kernel_alloc("cql_zone_map", 12);
  if (!out || !k) return 0;
  cqlcuda_kernel_set_arg_buffer(k, 0, column->buffer);
  cqlcuda_kernel_set_arg_buffer(k, 1, out);
  cqlcuda_kernel_set_arg_u64(k, 0, rows);
  cqlcuda_kernel_set_arg_u64(k, 1, (uint64_t)t | ((uint64_t)column->width << 32));
  cqlcuda_kernel_set_arg_u64(k, 2, column->base);
  cqlcuda_kernel_set_arg_u64(k, 3, ZONEMAP_LOG2);
  CqlBatch* b = cqlcuda_batch_begin(0, chunks * 16);
  cqlcuda_batch_kernel_execute(b, k, (uint32_t)(chunks < 0xffffffu ? chunks * 256 : 0xffffff00u), QE_GPU_WORKGROUP_SIZE);
  cqlcuda_batch_buffer_read(b, out, out_zone_map, chunks * 16);
  if (!cqlcuda_batch_end(b)) return 0;
  zone_summary(out_zone_map, chunks);
  return 1;
}

/* qe_zonemap_chunk_is_prunable (query_exec.c:13294-13304) */
static int chunk_prunable(uint32_t op, double target, double mn, double mx)
{
  if (mn > mx) return 0;   /* no values: never proven empty */
  switch (op)
  {
    case CQLOPS_CMP_EQ: return target < mn || target > mx;
    case CQLOPS_CMP_LT: return mn >= target;
    case CQLOPS_CMP_LE: return mn > target;
    case CQLOPS_CMP_GT: return mx <= target;
    case CQLOPS_CMP_GE: return mx < target;
    default: return 0;
  }
}

uint64_t cqlops_scan_ranges(const CqlColumn* columns, uint32_t column_count, const CqlLeaf* leaves, uint32_t leaf_count,
                            uint64_t* out_ranges, uint64_t max_ranges, uint32_t* out_skip_bits, int* out_use_skip,
                            uint64_t* out_pruned_rows)
{
  uint64_t rows = column_count ? columns[0].rows : 0;
  if (out_use_skip) *out_use_skip = 0;
  if (out_pruned_rows) *out_pruned_rows = 0;
  if (rows == 0 || max_ranges == 0) return 0;
  uint64_t chunks = (rows + CQLOPS_ZONEMAP_CHUNK_ROWS - 1) / CQLOPS_ZONEMAP_CHUNK_ROWS;
  /* the leaves a zone map can prove empty: numeric, one of = < <= > >=, a map present or implied.
     A zone-map leaf that its map's summary shows cannot prune any chunk is dropped at once; a leaf on a
     sequence (value = base + row, increasing when it does not wrap) keeps one interval of rows. */
  uint32_t usable[64];
  uint32_t usable_count = 0;
  uint64_t keep_lo = 0, keep_hi = rows;   /* rows the sequence leaves leave, [keep_lo, keep_hi) */
  int have_interval = 0;
  for (uint32_t l = 0; l < leaf_count && usable_count < 64; l++)
  {
    if (leaves[l].column >= column_count) continue;
    const CqlColumn* c = &columns[leaves[l].column];
    int numeric = c->type == CQLOPS_TYPE_U32 || c->type == CQLOPS_TYPE_I32 || c->type == CQLOPS_TYPE_F32 || c->type == CQLOPS_TYPE_F64;
    if (!numeric || leaves[l].op > CQLOPS_CMP_GE || c->rows != rows) continue;
    double t = leaves[l].target;
    if (c->width == 3)
    {
      double v0 = c->type == CQLOPS_TYPE_I32 ? (double)(int32_t)c->base : (double)c->base;
      double v1 = v0 + (double)(rows - 1);
      double top = c->type == CQLOPS_TYPE_I32 ? 2147483647.0 : 4294967295.0;
      if (v1 > top) continue;   /* wraps: no interval */
      /* rows r with v0 + r op t, as a real interval [lo, hi] of r, then whole rows */
      double lo = 0.0, hi = (double)(rows - 1);
      switch (leaves[l].op)
      {
        case CQLOPS_CMP_EQ: lo = ceil(t - v0); hi = floor(t - v0); break;
        case CQLOPS_CMP_LT: hi = ceil(t - v0) - 1.0; break;
        case CQLOPS_CMP_LE: hi = floor(t - v0); break;
        case CQLOPS_CMP_GT: lo = floor(t - v0) + 1.0; break;
        default: lo = ceil(t - v0); break;
      }
      if (lo < 0.0) lo = 0.0;
      if (hi > (double)(rows - 1)) hi = (double)(rows - 1);
      uint64_t a = lo > hi ? rows : (uint64_t)lo, b = lo > hi ? rows : (uint64_t)hi + 1;
      if (a > keep_lo) keep_lo = a;
      if (b < keep_hi) keep_hi = b;
      have_interval = 1;
      continue;
    }
    if (!c->zone_map || c->zone_map_chunks < chunks) continue;
    double max_min = c->zone_map[2 * chunks], min_max = c->zone_map[2 * chunks + 1];
    int can_prune;
    switch (leaves[l].op)
    {
      case CQLOPS_CMP_EQ: can_prune = t < max_min || t > min_max; break;
      case CQLOPS_CMP_LT: can_prune = max_min >= t; break;
      case CQLOPS_CMP_LE: can_prune = max_min > t; break;
      case CQLOPS_CMP_GT: can_prune = min_max <= t; break;
      default: can_prune = min_max < t; break;
    }
    if (can_prune) usable[usable_count++] = l;
  }
  if (have_interval && usable_count == 0)
  {
    /* sequence leaves only: the kept chunks are one run, no pass over the chunks */
    uint64_t z0 = keep_lo >= keep_hi ? chunks : keep_lo / CQLOPS_ZONEMAP_CHUNK_ROWS;
    uint64_t z1 = keep_lo >= keep_hi ? chunks : (keep_hi - 1) / CQLOPS_ZONEMAP_CHUNK_ROWS + 1;
    uint64_t first = z0 * CQLOPS_ZONEMAP_CHUNK_ROWS;
    uint64_t end = z1 * CQLOPS_ZONEMAP_CHUNK_ROWS < rows ? z1 * CQLOPS_ZONEMAP_CHUNK_ROWS : rows;
    uint64_t kept = z0 < z1 ? end - first : 0;
    if ((rows - kept) * 100 < rows * QE_SCAN_MIN_PRUNE_PERCENT)
    {
      out_ranges[0] = 0;
      out_ranges[1] = rows;
      return 1;
    }
    if (out_pruned_rows) *out_pruned_rows = rows - kept;
    if (!kept) return 0;
    out_ranges[0] = first;
    out_ranges[1] = end;
    return 1;
  }
  uint8_t* prunable = (usable_count || have_interval) ? (uint8_t*)calloc(chunks, 1) : NULL;
  uint64_t prunable_rows = 0;
  if (prunable)
  {
    if (have_interval)
    {
      /* chunks wholly outside the kept rows */
      uint64_t z0 = keep_lo >= keep_hi ? chunks : keep_lo / CQLOPS_ZONEMAP_CHUNK_ROWS;
      uint64_t z1 = keep_lo >= keep_hi ? chunks : (keep_hi - 1) / CQLOPS_ZONEMAP_CHUNK_ROWS + 1;
      memset(prunable, 1, z0);
      if (z1 < chunks) memset(prunable + z1, 1, chunks - z1);
    }
    for (uint32_t u = 0; u < usable_count; u++)
    {
      const CqlLeaf* leaf = &leaves[usable[u]];
      const double* zm = columns[leaf->column].zone_map;
      for (uint64_t z = 0; z < chunks; z++)
        if (!prunable[z] && chunk_prunable(leaf->op, leaf->target, zm[2 * z], zm[2 * z + 1])) prunable[z] = 1;
    }
    /* a short run of prunable chunks between two scanned ones is scanned too (:13442-13466) */
    uint64_t min_gap_chunks = QE_SCAN_MIN_PRUNE_GAP_ROWS / CQLOPS_ZONEMAP_CHUNK_ROWS;
    uint64_t gz = 0;
    while (gz < chunks)
    {
      if (!prunable[gz])
      {
        gz++;
        continue;
      }
      uint64_t gap_start = gz;
      while (gz < chunks && prunable[gz]) gz++;
      int interior = gap_start > 0 && gz < chunks;
      if (interior && gz - gap_start < min_gap_chunks) memset(prunable + gap_start, 0, gz - gap_start);
    }
    for (uint64_t z = 0; z < chunks; z++)
    {
      if (!prunable[z]) continue;
      uint64_t start = z * CQLOPS_ZONEMAP_CHUNK_ROWS;
      prunable_rows += (start + CQLOPS_ZONEMAP_CHUNK_ROWS < rows ? start + CQLOPS_ZONEMAP_CHUNK_ROWS : rows) - start;
    }
    /* pruning only pays when it removes a real share of the table (:13468-13476) */
    if (prunable_rows * 100 < rows * QE_SCAN_MIN_PRUNE_PERCENT)
    {
      memset(prunable, 0, chunks);
      prunable_rows = 0;
    }
  }
  if (!prunable || prunable_rows == 0)
  {
    free(prunable);
    out_ranges[0] = 0;
    out_ranges[1] = rows;
    return 1;
  }
  /* consecutive kept chunks merge into ranges (the whole table is one buffer: no size cap) */
  uint64_t range_count = 0, z = 0;
  int overflow = 0;
  while (z < chunks)
  {
    if (prunable[z])
    {
      z++;
      continue;
    }
    uint64_t start = z * CQLOPS_ZONEMAP_CHUNK_ROWS;
    while (z < chunks && !prunable[z]) z++;
    uint64_t end = z * CQLOPS_ZONEMAP_CHUNK_ROWS < rows ? z * CQLOPS_ZONEMAP_CHUNK_ROWS : rows;
    if (range_count < max_ranges)
    {
      out_ranges[2 * range_count] = start;
      out_ranges[2 * range_count + 1] = end;
    }
    else
      overflow = 1;
    range_count++;
  }
  if (out_pruned_rows) *out_pruned_rows = prunable_rows;
  /* one pass with a skip bitmap wins when the ranges cost more (:13513-13532) */
  if ((range_count > 1 && range_count * QE_SCAN_RANGE_COST_ROWS > rows) || overflow)
  {
    if (out_skip_bits && out_use_skip)
    {
      uint64_t words = (chunks + 31) / 32;
      memset(out_skip_bits, 0, words * 4);
      for (uint64_t zb = 0; zb < chunks; zb++)
        if (prunable[zb]) out_skip_bits[zb >> 5] |= 1u << (zb & 31);
      *out_use_skip = 1;
    }
    else if (out_pruned_rows)
      *out_pruned_rows = 0;
    free(prunable);
    out_ranges[0] = 0;
    out_ranges[1] = rows;
    return 1;
  }
  free(prunable);
  return range_count;
}
