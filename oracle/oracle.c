/*
 * oracle.c - CPU restatement of the reference's algorithms (TEST INFRASTRUCTURE ONLY: the checker
 * used by tests/, the smoke check and the bench's CPU-baseline leg; never part of the product).
 * Each function cites the reference source it restates.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define ORC_F64_MAX 1.7976931348623157e308

static uint32_t g_threads = 0;

void orc_set_threads(uint32_t n) { g_threads = n; }

uint32_t orc_threads(void)
{
  if (g_threads) return g_threads;
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  return n > 0 ? (uint32_t)n : 1u;
}

/* ---- a small parallel-for over task ids ---- */
typedef void (*orc_task_fn)(void* ctx, uint32_t task_id);
typedef struct
{
  orc_task_fn fn;
  void* ctx;
  uint32_t tasks;
  uint32_t next;
  pthread_mutex_t lock;
} orc_pool;

static void* orc_worker(void* p)
{
  orc_pool* pool = (orc_pool*)p;
  for (;;)
  {
    pthread_mutex_lock(&pool->lock);
    uint32_t id = pool->next++;
    pthread_mutex_unlock(&pool->lock);
    if (id >= pool->tasks) break;
    pool->fn(pool->ctx, id);
  }
  return NULL;
}

static void orc_parallel(uint32_t tasks, orc_task_fn fn, void* ctx)
{
  uint32_t workers = orc_threads();
  if (workers > tasks) workers = tasks;
  if (workers <= 1)
  {
    for (uint32_t i = 0; i < tasks; i++) fn(ctx, i);
    return;
  }
  orc_pool pool;
  pool.fn = fn;
  pool.ctx = ctx;
  pool.tasks = tasks;
  pool.next = 0;
  pthread_mutex_init(&pool.lock, NULL);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * workers);
  for (uint32_t i = 0; i < workers; i++) pthread_create(&th[i], NULL, orc_worker, &pool);
  for (uint32_t i = 0; i < workers; i++) pthread_join(th[i], NULL);
  free(th);
  pthread_mutex_destroy(&pool.lock);
}

void orc_parallel_for(uint32_t tasks, orc_task_fn fn, void* ctx) { orc_parallel(tasks, fn, ctx); }

/* ---- data ---- */

uint64_t orc_splitmix_draw(uint64_t seed, uint64_t k)
{
  uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

typedef struct
{
  uint32_t* out;
  uint64_t rows, seed, range;
  uint32_t per_row, index, tasks;
} fill_ctx;

static void fill_task(void* p, uint32_t id)
{
  fill_ctx* c = (fill_ctx*)p;
  uint64_t per = (c->rows + c->tasks - 1) / c->tasks;
  uint64_t lo = (uint64_t)id * per, hi = lo + per;
  if (hi > c->rows) hi = c->rows;
  for (uint64_t r = lo; r < hi; r++)
  {
    uint64_t v = orc_splitmix_draw(c->seed, r * c->per_row + c->index);
    c->out[r] = (uint32_t)(c->range ? v % c->range : v);
  }
}

void orc_fill_splitmix_u32(uint32_t* out, uint64_t rows, uint64_t seed, uint32_t per_row, uint32_t index, uint64_t range)
{
  fill_ctx c = { out, rows, seed, range, per_row, index, 64 };
  if (rows < 65536) c.tasks = 1;
  orc_parallel(c.tasks, fill_task, &c);
}

void orc_fill_closed_form(uint32_t* id, uint32_t* region, uint32_t* amount, uint32_t* needle_key, uint64_t rows)
{
  for (uint64_t i = 0; i < rows; i++)
  {
    if (id) id[i] = (uint32_t)(i + 1);
    if (region) region[i] = (uint32_t)(i % 50);
    if (amount) amount[i] = (uint32_t)(i % 10000);
    if (needle_key) needle_key[i] = (uint32_t)(i * 2654435761ull);
  }
}

/* ---- whole-column aggregates ---- */

static double widen(const void* values, uint32_t type, uint64_t i)
{
  switch (type)
  {
    case ORC_U32: return (double)((const uint32_t*)values)[i];
    case ORC_I32: return (double)((const int32_t*)values)[i];
    case ORC_U64: return (double)((const uint64_t*)values)[i];
    case ORC_I64: return (double)((const int64_t*)values)[i];
    case ORC_F32: return (double)((const float*)values)[i];
    default: return ((const double*)values)[i];
  }
}

typedef struct
{
  const void* values;
  uint32_t type;
  uint64_t base, rows, per;
  double* sum;
  double* mn;
  double* mx;
} agg_ctx;

/* QE_CHUNK_REDUCE_LOOP (query_exec.c:7472-7482) over one tp_divide_work range */
static void agg_task(void* p, uint32_t id)
{
  agg_ctx* c = (agg_ctx*)p;
  uint64_t lo = (uint64_t)id * c->per, hi = lo + c->per;
  if (lo > c->rows) lo = c->rows;
  if (hi > c->rows) hi = c->rows;
  double sum = 0.0, mn = ORC_F64_MAX, mx = -ORC_F64_MAX;
  for (uint64_t i = lo; i < hi; i++)
  {
    double v = widen(c->values, c->type, c->base + i);
    sum += v;
    if (v < mn) mn = v;
    if (v > mx) mx = v;
  }
  c->sum[id] = sum;
  c->mn[id] = mn;
  c->mx[id] = mx;
}

void orc_aggregate_global_cpu(const void* values, uint32_t type, uint64_t rows, uint32_t tasks_hint, double* out_sum, double* out_min,
                              double* out_max)
{
  double sum = 0.0, mn = ORC_F64_MAX, mx = -ORC_F64_MAX;
  const uint64_t chunk_rows = 67108864; /* QE_AGG_CHUNK_ROWS default (:9162) */
  uint32_t workers = tasks_hint ? tasks_hint : orc_threads();
  for (uint64_t start = 0; start < rows; start += chunk_rows)
  {
    uint64_t n = rows - start < chunk_rows ? rows - start : chunk_rows;
    uint64_t task_count = n / 65536;
    if (task_count > workers) task_count = workers;
    if (task_count < 1) task_count = 1;
    double* ts = (double*)malloc(sizeof(double) * task_count * 3);
    agg_ctx c = { values, type, start, n, (n + task_count - 1) / task_count, ts, ts + task_count, ts + 2 * task_count };
    orc_parallel((uint32_t)task_count, agg_task, &c);
    for (uint64_t t = 0; t < task_count; t++)
    {
      sum += c.sum[t];
      if (c.mn[t] < mn) mn = c.mn[t];
      if (c.mx[t] > mx) mx = c.mx[t];
    }
    free(ts);
  }
  *out_sum = sum;
  *out_min = mn;
  *out_max = mx;
}

void orc_aggregate_global_gpu_order(const void* values, uint32_t type, uint64_t rows, double* out_sum, double* out_min, double* out_max)
{
  const uint64_t chunk_rows = 16777216; /* qe_stream_chunk_rows (:2096-2099) */
  const uint32_t groups = 2048, wg = 256;
  const uint64_t stride = (uint64_t)groups * wg;
  double total = 0.0, tmin = ORC_F64_MAX, tmax = -ORC_F64_MAX;
  double* sh_sum = (double*)malloc(sizeof(double) * wg);
  double* sh_min = (double*)malloc(sizeof(double) * wg);
  double* sh_max = (double*)malloc(sizeof(double) * wg);
  uint32_t width = type == ORC_F64 ? 2 : 1;
  for (uint64_t start = 0; start < rows; start += chunk_rows)
  {
    uint64_t n = rows - start < chunk_rows ? rows - start : chunk_rows;
    uint64_t total_words = n * width, vec_count = total_words / 4, tail_start = vec_count * 4;
    for (uint32_t g = 0; g < groups; g++)
    {
      for (uint32_t tid = 0; tid < wg; tid++)
      {
        uint64_t t = (uint64_t)g * wg + tid;
        double acc = 0.0, mn = ORC_F64_MAX, mx = -ORC_F64_MAX;
        for (uint64_t i = t; i < vec_count; i += stride)
        {
          if (width == 1)
          {
            double v0 = widen(values, type, start + i * 4 + 0), v1 = widen(values, type, start + i * 4 + 1);
            double v2 = widen(values, type, start + i * 4 + 2), v3 = widen(values, type, start + i * 4 + 3);
            acc += (v0 + v1) + (v2 + v3);
            double a = v0 < v1 ? v0 : v1, b = v2 < v3 ? v2 : v3;
            double m = a < b ? a : b;
            mn = m < mn ? m : mn;
            a = v0 > v1 ? v0 : v1;
            b = v2 > v3 ? v2 : v3;
            m = a > b ? a : b;
            mx = m > mx ? m : mx;
          }
          else
          {
            double v0 = widen(values, type, start + i * 2 + 0), v1 = widen(values, type, start + i * 2 + 1);
            acc += v0 + v1;
            double a = v0 < v1 ? v0 : v1;
            mn = a < mn ? a : mn;
            a = v0 > v1 ? v0 : v1;
            mx = a > mx ? a : mx;
          }
        }
        if (width == 1)
        {
          if (t < total_words - tail_start)
          {
            double x = widen(values, type, start + tail_start + t);
            acc += x;
            mn = x < mn ? x : mn;
            mx = x > mx ? x : mx;
          }
        }
        else if (t == 0 && total_words > tail_start)
        {
          double x = widen(values, type, start + tail_start / 2);
          acc += x;
          mn = x < mn ? x : mn;
          mx = x > mx ? x : mx;
        }
        sh_sum[tid] = acc;
        sh_min[tid] = mn;
        sh_max[tid] = mx;
      }
      for (uint32_t step = 128; step > 0; step >>= 1)
      {
        for (uint32_t tid = 0; tid < step; tid++)
        {
          sh_sum[tid] += sh_sum[tid + step];
          sh_min[tid] = sh_min[tid + step] < sh_min[tid] ? sh_min[tid + step] : sh_min[tid];
          sh_max[tid] = sh_max[tid + step] > sh_max[tid] ? sh_max[tid + step] : sh_max[tid];
        }
      }
      total += sh_sum[0];
      tmin = sh_min[0] < tmin ? sh_min[0] : tmin;
      tmax = sh_max[0] > tmax ? sh_max[0] : tmax;
    }
  }
  free(sh_sum);
  free(sh_min);
  free(sh_max);
  *out_sum = total;
  *out_min = tmin;
  *out_max = tmax;
}

double orc_compensated_sum(const void* values, uint32_t type, uint64_t rows)
{
  double s = 0.0, c = 0.0;
  for (uint64_t i = 0; i < rows; i++)
  {
    double x = widen(values, type, i);
    double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
  }
  return s + c;
}

/* ---- scan + filter ---- */

static int leaf_match(const OrcLeaf* l, uint64_t row)
{
  double v = widen(l->values, l->type, row);
  switch (l->op)
  {
    case 0: return v == l->target;
    case 1: return v < l->target;
    case 2: return v <= l->target;
    case 3: return v > l->target;
    default: return v >= l->target;
  }
}

typedef struct
{
  const OrcLeaf* leaves;
  uint32_t leaf_count;
  uint64_t rows, per;
  uint64_t* counts;
  uint32_t** lists;
} scan_ctx;

static void scan_task(void* p, uint32_t id)
{
  scan_ctx* c = (scan_ctx*)p;
  uint64_t lo = (uint64_t)id * c->per, hi = lo + c->per;
  if (lo > c->rows) lo = c->rows;
  if (hi > c->rows) hi = c->rows;
  uint64_t n = 0;
  for (uint64_t r = lo; r < hi; r++)
  {
    int ok = 1;
    for (uint32_t l = 0; l < c->leaf_count && ok; l++) ok = leaf_match(&c->leaves[l], r);
    if (ok)
    {
      if (c->lists && c->lists[id]) c->lists[id][n] = (uint32_t)r;
      n++;
    }
  }
  c->counts[id] = n;
}

uint64_t orc_scan_and(const OrcLeaf* leaves, uint32_t leaf_count, uint64_t rows, uint32_t* out_rows, uint64_t cap)
{
  uint32_t tasks = orc_threads();
  if (rows < 65536) tasks = 1;
  scan_ctx c;
  c.leaves = leaves;
  c.leaf_count = leaf_count;
  c.rows = rows;
  c.per = (rows + tasks - 1) / tasks;
  c.counts = (uint64_t*)calloc(tasks, sizeof(uint64_t));
  c.lists = NULL;
  if (out_rows && cap)
  {
    c.lists = (uint32_t**)calloc(tasks, sizeof(uint32_t*));
    for (uint32_t t = 0; t < tasks; t++) c.lists[t] = (uint32_t*)malloc(sizeof(uint32_t) * (c.per ? c.per : 1));
  }
  orc_parallel(tasks, scan_task, &c);
  uint64_t total = 0;
  for (uint32_t t = 0; t < tasks; t++)
  {
    if (c.lists)
    {
      for (uint64_t i = 0; i < c.counts[t] && total + i < cap; i++) out_rows[total + i] = c.lists[t][i];
      free(c.lists[t]);
    }
    total += c.counts[t];
  }
  free(c.lists);
  free(c.counts);
  return total;
}

/* ---- dense GROUP BY ---- */

void orc_group_dense(const uint32_t* key, uint32_t key_type, uint64_t rows, int64_t min_key, uint64_t groups, uint32_t expr_count,
                     const uint32_t* funcs, const uint32_t* const* args, const uint32_t* arg_types, uint64_t* out_counts,
                     int64_t* out_sums, int64_t* out_mins, int64_t* out_maxs)
{
  for (uint64_t g = 0; g < groups; g++)
  {
    out_counts[g] = 0;
    for (uint32_t e = 0; e < expr_count; e++)
    {
      out_sums[g * expr_count + e] = 0;
      out_mins[g * expr_count + e] = 2147483647;
      out_maxs[g * expr_count + e] = -2147483648ll;
    }
  }
  for (uint64_t r = 0; r < rows; r++)
  {
    int64_t k = key_type == ORC_I32 ? (int64_t)(int32_t)key[r] : (int64_t)key[r];
    int64_t g = k - min_key;
    if (g < 0 || (uint64_t)g >= groups) continue;
    out_counts[g] += 1;
    for (uint32_t e = 0; e < expr_count; e++)
    {
      uint32_t f = funcs[e];
      if (f == 0) continue;
      uint32_t w = args[e][r];
      int64_t* s = &out_sums[g * expr_count + e];
      if (f == 1 || f == 2)
      {
        uint64_t add = arg_types[e] == ORC_I32 ? (uint64_t)(int64_t)(int32_t)w : (uint64_t)w;
        *s = (int64_t)((uint64_t)*s + add);
      }
      else if (f == 3)
      {
        int64_t v = (int64_t)(int32_t)w;
        if (v < out_mins[g * expr_count + e]) out_mins[g * expr_count + e] = v;
      }
      else if (f == 4)
      {
        int64_t v = (int64_t)(int32_t)w;
        if (v > out_maxs[g * expr_count + e]) out_maxs[g * expr_count + e] = v;
      }
    }
  }
}

/* The reference hashes its keys with qe_aggregate_hash_key; the table order only affects speed,
   the groups come out in first-appearance order either way. This restatement hashes the key word. */
static uint64_t key_hash(uint32_t k)
{
  uint64_t h = (uint64_t)k * 0x9E3779B97F4A7C15ull;
  return h ^ (h >> 29);
}

uint64_t orc_group_cpu_reduce(const uint32_t* key, uint64_t rows, uint32_t expr_count, const uint32_t* const* args, uint64_t max_groups,
                              uint32_t* out_keys, uint64_t* out_counts, double* out_sums, double* out_mins, double* out_maxs)
{
  uint64_t table_size = 16;
  while (table_size < max_groups * 2) table_size <<= 1;
  uint32_t* table = (uint32_t*)malloc(sizeof(uint32_t) * table_size);
  for (uint64_t i = 0; i < table_size; i++) table[i] = 0xffffffffu;
  uint64_t group_count = 0;
  for (uint64_t r = 0; r < rows; r++)
  {
    uint64_t slot = key_hash(key[r]) & (table_size - 1);
    uint64_t g;
    for (;;)
    {
      uint32_t occ = table[slot];
      if (occ == 0xffffffffu)
      {
        if (group_count >= max_groups)
        {
          free(table);
          return 0;
        }
        g = group_count++;
        table[slot] = (uint32_t)g;
        out_keys[g] = key[r];
        out_counts[g] = 0;
        for (uint32_t e = 0; e < expr_count; e++)
        {
          out_sums[g * expr_count + e] = 0.0;
          out_mins[g * expr_count + e] = 1.0e300;
          out_maxs[g * expr_count + e] = -1.0e300;
        }
        break;
      }
      if (out_keys[occ] == key[r])
      {
        g = occ;
        break;
      }
      slot = (slot + 1) & (table_size - 1);
    }
    out_counts[g] += 1;
    for (uint32_t e = 0; e < expr_count; e++)
    {
      double v = args[e] ? (double)args[e][r] : 0.0;
      out_sums[g * expr_count + e] += v;
      if (v < out_mins[g * expr_count + e]) out_mins[g * expr_count + e] = v;
      if (v > out_maxs[g * expr_count + e]) out_maxs[g * expr_count + e] = v;
    }
  }
  free(table);
  return group_count;
}

/* ---- scan bytecode ---- */

static double slot_value(const void* const* data, const uint32_t* types, uint32_t slot, uint64_t row)
{
  const void* p = data[slot];
  switch (types[slot])
  {
    case 1: case 12: return (double)((const uint32_t*)p)[row];
    case 2:
    {
      uint64_t v = ((const uint64_t*)p)[row];
      return (double)(uint32_t)(v >> 32) * 4294967296.0 + (double)(uint32_t)v;
    }
    case 3: return (double)((const float*)p)[row];
    case 4: return ((const double*)p)[row];
    case 6: return (double)((const uint8_t*)p)[row];
    case 7: case 9: return (double)((const int32_t*)p)[row];
    default:
    {
      uint64_t v = ((const uint64_t*)p)[row];
      double u = (double)(uint32_t)(v >> 32) * 4294967296.0 + (double)(uint32_t)v;
      return (v >> 63) ? u - 18446744073709551616.0 : u;
    }
  }
}

/* qe_str8_compare-style three-way compare of a row's string with a constant (scan_filter.comp:185-207) */
static int str_cmp3(const void* const* data, uint32_t slot, uint64_t row, const uint8_t* c, uint32_t len)
{
  const uint8_t* bytes = (const uint8_t*)data[slot];
  const uint64_t* offs = (const uint64_t*)data[slot + 1];
  uint64_t s = offs[row], e = offs[row + 1], n = e - s, m = n < len ? n : len;
  for (uint64_t i = 0; i < m; i++)
  {
    if (bytes[s + i] != c[i]) return bytes[s + i] < c[i] ? -1 : 1;
  }
  return n < len ? -1 : (n > len ? 1 : 0);
}

static int str_contains(const void* const* data, uint32_t slot, uint64_t row, const uint8_t* c, uint32_t len)
{
  const uint8_t* bytes = (const uint8_t*)data[slot];
  const uint64_t* offs = (const uint64_t*)data[slot + 1];
  uint64_t s = offs[row], n = offs[row + 1] - s;
  if (len == 0) return 1;
  for (uint64_t i = 0; i + len <= n; i++)
    if (memcmp(bytes + s + i, c, len) == 0) return 1;
  return 0;
}

#define FUZZY_MAX_NEEDLE 64u          /* QE_FUZZY_MAX_NEEDLE_LEN, scan_filter.comp:35 */
#define FUZZY_MAX_STRING 1048576u     /* MAX_SANE_STRING_LEN, scan_filter.comp:205 */

/* trigram_similarity (scan_filter.comp:236-290): the shared n-grams of the row and the needle, each needle
   gram used once, the first unused match taken, over the union of the two gram counts */
static double str_trigram(const void* const* data, uint32_t slot, uint64_t row, const uint8_t* c, uint32_t clen, uint32_t n)
{
  const uint8_t* bytes = (const uint8_t*)data[slot];
  const uint64_t* offs = (const uint64_t*)data[slot + 1];
  uint64_t s = offs[row], len = offs[row + 1] - s;
  if (len < n || clen < n)
  {
    if (len != clen) return 0.0;
    return memcmp(bytes + s, c, len) == 0 ? 1.0 : 0.0;
  }
  if (len > FUZZY_MAX_STRING) return 0.0;
  uint32_t needle_grams = clen - n + 1 < FUZZY_MAX_NEEDLE ? clen - n + 1 : FUZZY_MAX_NEEDLE;
  uint8_t used[FUZZY_MAX_NEEDLE] = { 0 };
  uint64_t hay_grams = len - n + 1, shared = 0;
  for (uint64_t i = 0; i < hay_grams; i++)
    for (uint32_t j = 0; j < needle_grams; j++)
    {
      if (used[j]) continue;
      if (memcmp(bytes + s + i, c + j, n) == 0)
      {
        used[j] = 1;
        shared++;
        break;
      }
    }
  uint64_t uni = hay_grams + needle_grams - shared;
  return uni == 0 ? 0.0 : (double)shared / (double)uni;
}

/* edit_distance (scan_filter.comp:292-323): the Levenshtein distance to the first 64 bytes of the needle,
   one rolling row */
static double str_edit_distance(const void* const* data, uint32_t slot, uint64_t row, const uint8_t* c, uint32_t clen)
{
  const uint8_t* bytes = (const uint8_t*)data[slot];
  const uint64_t* offs = (const uint64_t*)data[slot + 1];
  uint64_t s = offs[row], len = offs[row + 1] - s;
  if (len > FUZZY_MAX_STRING) return (double)FUZZY_MAX_STRING;
  uint32_t m = clen < FUZZY_MAX_NEEDLE ? clen : FUZZY_MAX_NEEDLE;
  uint32_t dp[FUZZY_MAX_NEEDLE + 1];
  for (uint32_t j = 0; j <= m; j++) dp[j] = j;
  for (uint64_t i = 1; i <= len; i++)
  {
    uint32_t diag = dp[0];
    dp[0] = (uint32_t)i;
    for (uint32_t j = 1; j <= m; j++)
    {
      uint32_t keep = dp[j];
      uint32_t cost = bytes[s + i - 1] == c[j - 1] ? 0u : 1u;
      uint32_t best = dp[j] + 1u;
      if (dp[j - 1] + 1u < best) best = dp[j - 1] + 1u;
      if (diag + cost < best) best = diag + cost;
      dp[j] = best;
      diag = keep;
    }
  }
  return (double)dp[m];
}

static uint64_t eval_program(const uint32_t* words, uint32_t word_count, const uint32_t* consts, const uint8_t* str_pool,
                             const void* const* slot_data, const uint32_t* slot_types, uint64_t rows, uint8_t* out_match, double* out_score)
{
  uint64_t count = 0;
  double stack[64];
  for (uint64_t row = 0; row < rows; row++)
  {
    int sp = 0;
    uint32_t ip = 0;
    int ok = 1;
    double score = 0.0;   /* the last fuzzy score of the row, as the scan outputs it */
    while (ok && ip < word_count)
    {
      uint32_t op = words[ip++];
      if (op == 13) break;
      switch (op)
      {
        case 0: stack[sp++] = 1.0; break;
        case 14: stack[sp++] = 0.0; break;
        case 1:
        {
          uint32_t operand = words[ip++];
          uint32_t slot = operand & 0xffu;
          uint32_t saved = slot_types[slot];
          uint32_t types_local[10];
          memcpy(types_local, slot_types, sizeof(types_local));
          types_local[slot] = (operand >> 8) & 0xffu;
          (void)saved;
          stack[sp++] = slot_value(slot_data, types_local, slot, row);
          break;
        }
        case 2:
        {
          uint32_t k = words[ip++];
          uint64_t bits = ((uint64_t)consts[2 * k + 1] << 32) | consts[2 * k];
          double v;
          memcpy(&v, &bits, sizeof(v));
          stack[sp++] = v;
          break;
        }
        case 3: case 4: case 5: case 6: case 7: case 8: case 9: case 10:
        {
          double b = stack[--sp], a = stack[--sp];
          int r = op == 3 ? a == b : op == 4 ? a != b : op == 5 ? a < b : op == 6 ? a > b : op == 7 ? a <= b : op == 8 ? a >= b
                : op == 9 ? (a != 0.0 && b != 0.0) : (a != 0.0 || b != 0.0);
          stack[sp++] = r ? 1.0 : 0.0;
          break;
        }
        case 11: case 12: case 17: case 18: case 19: case 20: case 21:
        {
          uint32_t slot = words[ip], wo = words[ip + 1], len = words[ip + 2];
          ip += 3;
          const uint8_t* c = str_pool + (uint64_t)wo * 4;
          int r;
          if (op == 12) r = str_contains(slot_data, slot, row, c, len);
          else
          {
            int t = str_cmp3(slot_data, slot, row, c, len);
            r = op == 11 ? t == 0 : op == 17 ? t != 0 : op == 18 ? t < 0 : op == 19 ? t > 0 : op == 20 ? t <= 0 : t >= 0;
          }
          stack[sp++] = r ? 1.0 : 0.0;
          break;
        }
        case 15: case 16:
        {
          uint32_t slot = words[ip], wo = words[ip + 1], len = words[ip + 2];
          ip += 3;
          const uint8_t* c = str_pool + (uint64_t)wo * 4;
          double v = op == 15 ? str_trigram(slot_data, slot, row, c, len, 3) : str_edit_distance(slot_data, slot, row, c, len);
          /* the scan reports a similarity as an f32 and a distance as an integer */
          score = op == 15 ? (double)(float)v : (double)(uint32_t)v;
          stack[sp++] = v;
          break;
        }
        default: ok = 0; break;
      }
      if (sp >= 63) ok = 0;
    }
    int m = sp > 0 && stack[sp - 1] != 0.0;
    if (out_match) out_match[row] = (uint8_t)m;
    if (out_score) out_score[row] = score;
    count += (uint64_t)m;
  }
  return count;
}

uint64_t orc_eval_program(const uint32_t* words, uint32_t word_count, const uint32_t* consts, const uint8_t* str_pool,
                          const void* const* slot_data, const uint32_t* slot_types, uint64_t rows, uint8_t* out_match)
{
  return eval_program(words, word_count, consts, str_pool, slot_data, slot_types, rows, out_match, NULL);
}

uint64_t orc_eval_program_scored(const uint32_t* words, uint32_t word_count, const uint32_t* consts, const uint8_t* str_pool,
                                 const void* const* slot_data, const uint32_t* slot_types, uint64_t rows, uint8_t* out_match, double* out_score)
{
  return eval_program(words, word_count, consts, str_pool, slot_data, slot_types, rows, out_match, out_score);
}

/* ---- a batch of WHERE programs over one table: COUNT(*) and SUM of a column per program ----
   The same interpreter as eval_program, run a block of rows at a time: every opcode of a program acts on a
   whole block (a stack of blocks of doubles), so one pass over the table serves every program of the
   batch while the block is in cache. Threads take ranges of rows; each range keeps a Neumaier
   compensated sum per program, and the ranges are folded in order the same way. Numeric opcodes only
   (the batched shared scan takes no string comparisons). Returns 0 on an opcode it does not take. */
#define BATCH_BLOCK 1024u
#define BATCH_STACK 24
typedef struct
{
  uint32_t programs;
  const uint32_t* const* words;
  const uint32_t* word_counts;
  const uint32_t* const* consts;
  const void* const* slot_data;    /* programs x 10 */
  const uint32_t* slot_types;      /* programs x 10 */
  const void* const* sum_data;     /* programs: the summed column or NULL */
  const uint32_t* sum_types;
  uint64_t rows;
  uint64_t rows_per_task;
  uint64_t* counts;                /* tasks x programs */
  double* sums;                    /* tasks x programs x 2: sum, compensation */
  int failed;
} BatchCtx;

static void batch_load(double* out, const void* p, uint32_t type, uint64_t first, uint32_t n)
{
  switch (type)
  {
    case 1: case 12: for (uint32_t i = 0; i < n; i++) out[i] = (double)((const uint32_t*)p)[first + i]; break;
    case 3: for (uint32_t i = 0; i < n; i++) out[i] = (double)((const float*)p)[first + i]; break;
    case 4: for (uint32_t i = 0; i < n; i++) out[i] = ((const double*)p)[first + i]; break;
    case 6: for (uint32_t i = 0; i < n; i++) out[i] = (double)((const uint8_t*)p)[first + i]; break;
    case 7: case 9: for (uint32_t i = 0; i < n; i++) out[i] = (double)((const int32_t*)p)[first + i]; break;
    default:
    {
      const void* data[1] = {p};
      uint32_t types[1] = {type};
      for (uint32_t i = 0; i < n; i++) out[i] = slot_value(data, types, 0, first + i);
    }
  }
}

static void batch_task(void* arg, uint32_t task)
{
  BatchCtx* x = (BatchCtx*)arg;
  uint64_t lo = (uint64_t)task * x->rows_per_task, hi = lo + x->rows_per_task;
  if (hi > x->rows) hi = x->rows;
  double* stack = (double*)malloc(sizeof(double) * BATCH_BLOCK * (BATCH_STACK + 1));
  double* sumv = stack + (size_t)BATCH_BLOCK * BATCH_STACK;
  uint64_t* counts = x->counts + (size_t)task * x->programs;
  double* sums = x->sums + (size_t)task * x->programs * 2;
  for (uint64_t first = lo; first < hi; first += BATCH_BLOCK)
  {
    uint32_t n = (uint32_t)((hi - first) < BATCH_BLOCK ? (hi - first) : BATCH_BLOCK);
    for (uint32_t q = 0; q < x->programs; q++)
    {
      const uint32_t* w = x->words[q];
      const uint32_t* k = x->consts[q];
      uint32_t wc = x->word_counts[q], ip = 0;
      int sp = 0;
      while (ip < wc)
      {
        uint32_t op = w[ip++];
        if (op == 13) break;
        if (sp >= BATCH_STACK - 1) { x->failed = 1; break; }
        double* top = stack + (size_t)sp * BATCH_BLOCK;
        if (op == 0 || op == 14 || op == 2)
        {
          double v = op == 0 ? 1.0 : 0.0;
          if (op == 2)
          {
            uint32_t c = w[ip++];
            uint64_t bits = ((uint64_t)k[2 * c + 1] << 32) | k[2 * c];
            memcpy(&v, &bits, sizeof(v));
          }
          for (uint32_t i = 0; i < n; i++) top[i] = v;
          sp++;
        }
        else if (op == 1)
        {
          uint32_t operand = w[ip++], slot = operand & 0xffu;
          batch_load(top, x->slot_data[(size_t)q * 10 + slot], (operand >> 8) & 0xffu, first, n);
          sp++;
        }
        else if (op >= 3 && op <= 10 && sp >= 2)
        {
          double* b = top - BATCH_BLOCK;
          double* a = b - BATCH_BLOCK;
          switch (op)
          {
            case 3: for (uint32_t i = 0; i < n; i++) a[i] = a[i] == b[i] ? 1.0 : 0.0; break;
            case 4: for (uint32_t i = 0; i < n; i++) a[i] = a[i] != b[i] ? 1.0 : 0.0; break;
            case 5: for (uint32_t i = 0; i < n; i++) a[i] = a[i] < b[i] ? 1.0 : 0.0; break;
            case 6: for (uint32_t i = 0; i < n; i++) a[i] = a[i] > b[i] ? 1.0 : 0.0; break;
            case 7: for (uint32_t i = 0; i < n; i++) a[i] = a[i] <= b[i] ? 1.0 : 0.0; break;
            case 8: for (uint32_t i = 0; i < n; i++) a[i] = a[i] >= b[i] ? 1.0 : 0.0; break;
            case 9: for (uint32_t i = 0; i < n; i++) a[i] = (a[i] != 0.0 && b[i] != 0.0) ? 1.0 : 0.0; break;
            default: for (uint32_t i = 0; i < n; i++) a[i] = (a[i] != 0.0 || b[i] != 0.0) ? 1.0 : 0.0; break;
          }
          sp--;
        }
        else { x->failed = 1; break; }
      }
      if (sp <= 0) { x->failed = 1; continue; }
      const double* m = stack + (size_t)(sp - 1) * BATCH_BLOCK;
      uint64_t c = 0;
      for (uint32_t i = 0; i < n; i++) c += m[i] != 0.0;
      counts[q] += c;
      if (x->sum_data[q] && c)
      {
        batch_load(sumv, x->sum_data[q], x->sum_types[q], first, n);
        double s = sums[2 * q], comp = sums[2 * q + 1];
        for (uint32_t i = 0; i < n; i++)
        {
          if (m[i] == 0.0) continue;
          double v = sumv[i], t = s + v;
          comp += fabs(s) >= fabs(v) ? (s - t) + v : (v - t) + s;
          s = t;
        }
        sums[2 * q] = s;
        sums[2 * q + 1] = comp;
      }
    }
  }
  free(stack);
}

int orc_batch_count_sum(uint32_t programs, const uint32_t* const* words, const uint32_t* word_counts, const uint32_t* const* consts,
                        const void* const* slot_data, const uint32_t* slot_types, const void* const* sum_data, const uint32_t* sum_types,
                        uint64_t rows, uint64_t* out_count, double* out_sum)
{
  BatchCtx x;
  x.programs = programs;
  x.words = words;
  x.word_counts = word_counts;
  x.consts = consts;
  x.slot_data = slot_data;
  x.slot_types = slot_types;
  x.sum_data = sum_data;
  x.sum_types = sum_types;
  x.rows = rows;
  x.rows_per_task = 1u << 20;
  x.failed = 0;
  uint32_t tasks = (uint32_t)((rows + x.rows_per_task - 1) / x.rows_per_task);
  if (tasks == 0) tasks = 1;
  x.counts = (uint64_t*)calloc((size_t)tasks * programs, sizeof(uint64_t));
  x.sums = (double*)calloc((size_t)tasks * programs * 2, sizeof(double));
  orc_parallel(tasks, batch_task, &x);
  for (uint32_t q = 0; q < programs; q++)
  {
    uint64_t c = 0;
    double s = 0.0, comp = 0.0;
    for (uint32_t t = 0; t < tasks; t++)
    {
      c += x.counts[(size_t)t * programs + q];
      const double* part = x.sums + ((size_t)t * programs + q) * 2;
      for (int h = 0; h < 2; h++)
      {
        double v = part[h], u = s + v;
        comp += fabs(s) >= fabs(v) ? (s - u) + v : (v - u) + s;
        s = u;
      }
    }
    out_count[q] = c;
    out_sum[q] = s + comp;
  }
  free(x.counts);
  free(x.sums);
  return !x.failed;
}
