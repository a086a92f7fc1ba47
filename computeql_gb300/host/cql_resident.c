/*
 * cql_resident.c - the resident chunk cache: device copies of host column chunks kept between queries
 * (QE_ResidentCache, src/query_exec/query_exec.c:1679-1970).
 *
 * A chunk is found by (column, write generation, first row, rows, stored width). A hit hands back the
 * cached buffer; a miss makes room within the budget and copies the rows in. Room is made the
 * reference's way: first the entries used only once (a scan that passed through once), the most recent of
 * them first, then the least recently used of the rest; pinned entries are never taken. A column written
 * since (a new generation) makes its entries unusable, and they are freed on sight. The budget is a share
 * of the device's memory, never more than the memory the driver reports reachable, less a reserve. The
 * allocator's eviction hook frees entries when another allocation does not fit.
 *
 * The memory operations are callbacks, so the policy runs the same over device buffers (the default: the
 * cqlcuda backend) and over any other allocator a caller provides. No callback runs under the cache's lock:
 * the backend calls the eviction hook while it holds its own, so the cache takes its lock inside the
 * backend's and never the other way round; freed buffers are collected under the lock and released after.
 */
#include "cqlops.h"
#include "cql_ops_internal.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define RESIDENT_MAX_ENTRIES 4096
#define RESIDENT_RESERVE (512ull << 20)
#define RESIDENT_BUDGET_PERCENT 70

typedef struct
{
  int used, ready;
  uint64_t column_uid, generation, row_start, rows;
  uint32_t width;
  void* buffer;
  uint64_t bytes;
  uint64_t last_use;
  uint32_t uses, pins;
} ResidentChunk;

struct CqlResident
{
  pthread_mutex_t lock;
  ResidentChunk entries[RESIDENT_MAX_ENTRIES];
  uint64_t tick, bytes_in_use, entry_count, hit_bytes, miss_bytes, evicted_bytes;
  uint64_t budget_bytes;   /* 0: the share of device memory */
  CqlResidentOps ops;
};

static CqlResident* g_hooked = NULL;   /* the cache the backend's eviction hook frees from */

static uint64_t budget(CqlResident* r)
{
  uint64_t total = r->ops.total_memory ? r->ops.total_memory(r->ops.ctx) : 0;
  uint64_t b = total / 100 * RESIDENT_BUDGET_PERCENT;
  if (r->budget_bytes && (r->budget_bytes < b || !total)) b = r->budget_bytes;
  /* other buffers, the driver and other processes use device memory too */
  if (r->ops.free_memory)
  {
    uint64_t reachable = r->bytes_in_use + r->ops.free_memory(r->ops.ctx);
    reachable = reachable > RESIDENT_RESERVE ? reachable - RESIDENT_RESERVE : 0;
    if (reachable < b) b = reachable;
  }
  return b;
}

/* buffers taken out of the cache under its lock, released after it */
typedef struct
{
  void* items[64];
  uint32_t n;
} Doomed;

static void doom_release(CqlResident* r, Doomed* d)
{
  for (uint32_t i = 0; i < d->n; i++) r->ops.release(r->ops.ctx, d->items[i]);
  d->n = 0;
}

/* unlinks an entry; its buffer goes to `d` (released at once when `d` is full, which only the
   unlocked paths allow) */
static void unlink_entry(CqlResident* r, ResidentChunk* e, Doomed* d)
{
  if (e->buffer) d->items[d->n++] = e->buffer;
  r->bytes_in_use -= e->bytes < r->bytes_in_use ? e->bytes : r->bytes_in_use;
  r->entry_count -= 1;
  memset(e, 0, sizeof(*e));
}

/* entries used once go first (the most recent of them), then the least recently used */
static ResidentChunk* pick_victim(CqlResident* r)
{
  ResidentChunk *probation = NULL, *lru = NULL;
  for (int i = 0; i < RESIDENT_MAX_ENTRIES; i++)
  {
    ResidentChunk* e = &r->entries[i];
    if (!e->used || e->pins > 0 || !e->ready) continue;
    if (e->uses <= 1)
    {
      if (!probation || e->last_use > probation->last_use) probation = e;
    }
    else if (!lru || e->last_use < lru->last_use)
      lru = e;
  }
  return probation ? probation : lru;
}

/* evicts until `wanted` bytes are freed, none can be or `d` is full; returns the bytes freed */
static uint64_t evict_locked(CqlResident* r, uint64_t wanted, Doomed* d)
{
  uint64_t freed = 0;
  while (freed < wanted && d->n < 64)
  {
    ResidentChunk* v = pick_victim(r);
    if (!v) break;
    freed += v->bytes;
    r->evicted_bytes += v->bytes;
    unlink_entry(r, v, d);
  }
  return freed;
}

static uint64_t evict(CqlResident* r, uint64_t wanted)
{
  uint64_t freed = 0;
  for (;;)
  {
    Doomed d = { { 0 }, 0 };
    pthread_mutex_lock(&r->lock);
    uint64_t got = evict_locked(r, wanted - freed, &d);
    pthread_mutex_unlock(&r->lock);
    doom_release(r, &d);
    freed += got;
    if (!got || freed >= wanted) return freed;
  }
}

/* the backend calls this when an allocation does not fit (g_gpu_evict_hook) */
static uint64_t backend_evict_hook(uint64_t wanted)
{
  CqlResident* r = g_hooked;
  return r ? evict(r, wanted) : 0;
}

/* ---- the cqlcuda backend as the allocator ---- */

static void* dev_alloc(void* ctx, uint64_t bytes)
{
  (void)ctx;
  return cqlcuda_buffer_alloc(bytes, CQLCUDA_BUFFER_READ_WRITE, NULL);
}

static int dev_copy(void* ctx, void* buffer, const void* host, uint64_t bytes)
{
  (void)ctx;
  CqlBatch* b = cqlcuda_batch_begin(bytes, 0);
  cqlcuda_batch_buffer_write(b, (CqlBuffer*)buffer, host, bytes);
  return cqlcuda_batch_end(b);
}

static void dev_release(void* ctx, void* buffer)
{
  (void)ctx;
  cqlcuda_buffer_release((CqlBuffer*)buffer);
}

static uint64_t dev_total(void* ctx)
{
  (void)ctx;
  return cqlcuda_device_total_memory();
}

static uint64_t dev_free(void* ctx)
{
  (void)ctx;
  return cqlcuda_device_free_memory();
}

CqlResident* cqlops_resident_create(uint64_t budget_bytes, const CqlResidentOps* ops)
{
  CqlResident* r = (CqlResident*)calloc(1, sizeof(CqlResident));
  if (!r) return NULL;
  pthread_mutex_init(&r->lock, NULL);
  r->budget_bytes = budget_bytes;
  if (ops) r->ops = *ops;
  else
  {
    r->ops.alloc = dev_alloc;
    r->ops.copy = dev_copy;
    r->ops.release = dev_release;
    r->ops.total_memory = dev_total;
    r->ops.free_memory = dev_free;
    r->ops.ctx = NULL;
    /* the backend frees from this cache when an allocation does not fit (qe_resident_acquire sets
       g_gpu_evict_hook the same way) */
    g_hooked = r;
    cqlcuda_set_evict_hook(backend_evict_hook);
  }
  return r;
}

void cqlops_resident_destroy(CqlResident* r)
{
  if (!r) return;
  if (g_hooked == r)
  {
    cqlcuda_set_evict_hook(NULL);
    g_hooked = NULL;
  }
  for (int i = 0; i < RESIDENT_MAX_ENTRIES; i++)
    if (r->entries[i].used && r->entries[i].buffer) r->ops.release(r->ops.ctx, r->entries[i].buffer);
  pthread_mutex_destroy(&r->lock);
  free(r);
}

void* cqlops_resident_acquire(CqlResident* r, uint64_t column_uid, uint64_t generation, const void* host_rows, uint64_t row_start, uint64_t rows,
                              uint32_t width, int* out_hit)
{
  if (out_hit) *out_hit = 0;
  if (!r) return NULL;
  uint64_t bytes = rows * width;
  uint64_t b = budget(r);   /* asks the allocator for free memory: outside the lock */
  Doomed d = { { 0 }, 0 };
  pthread_mutex_lock(&r->lock);
  ResidentChunk* free_slot = NULL;
  for (int i = 0; i < RESIDENT_MAX_ENTRIES; i++)
  {
    ResidentChunk* e = &r->entries[i];
    if (!e->used)
    {
      if (!free_slot) free_slot = e;
      continue;
    }
    if (e->column_uid != column_uid) continue;
    if (e->generation != generation)
    {
      /* the column has been written since: nothing in this entry can be used again */
      if (e->pins == 0 && e->ready && d.n < 64)
      {
        unlink_entry(r, e, &d);
        if (!free_slot) free_slot = e;
      }
      continue;
    }
    if (e->ready && e->row_start == row_start && e->rows == rows && e->width == width)
    {
      r->tick++;
      e->last_use = r->tick;
      e->uses++;
      e->pins++;
      r->hit_bytes += bytes;
      void* buf = e->buffer;
      pthread_mutex_unlock(&r->lock);
      doom_release(r, &d);
      if (out_hit) *out_hit = 1;
      return buf;
    }
  }
  int fits = free_slot && bytes && bytes <= b && host_rows;
  if (fits && r->bytes_in_use + bytes > b)
  {
    uint64_t over = r->bytes_in_use + bytes - b;
    fits = evict_locked(r, over, &d) >= over;
  }
  if (!fits)
  {
    pthread_mutex_unlock(&r->lock);
    doom_release(r, &d);
    return NULL;
  }
  /* the slot is held (pinned, not ready: no one finds it, no one evicts it) while the buffer is made */
  r->tick++;
  free_slot->used = 1;
  free_slot->ready = 0;
  free_slot->column_uid = column_uid;
  free_slot->generation = generation;
  free_slot->row_start = row_start;
  free_slot->rows = rows;
  free_slot->width = width;
  free_slot->buffer = NULL;
  free_slot->bytes = bytes;
  free_slot->last_use = r->tick;
  free_slot->uses = 1;
  free_slot->pins = 1;
  r->bytes_in_use += bytes;
  r->entry_count++;
  r->miss_bytes += bytes;
  pthread_mutex_unlock(&r->lock);
  doom_release(r, &d);
  void* buf = r->ops.alloc(r->ops.ctx, bytes);
  int copied = buf && r->ops.copy(r->ops.ctx, buf, host_rows, bytes);
  pthread_mutex_lock(&r->lock);
  if (copied)
  {
    free_slot->buffer = buf;
    free_slot->ready = 1;
  }
  else
  {
    free_slot->buffer = NULL;
    unlink_entry(r, free_slot, &d);
  }
  pthread_mutex_unlock(&r->lock);
  if (!copied && buf) r->ops.release(r->ops.ctx, buf);
  return copied ? buf : NULL;
}

void cqlops_resident_release(CqlResident* r, const void* buffer)
{
  if (!r || !buffer) return;
  pthread_mutex_lock(&r->lock);
  for (int i = 0; i < RESIDENT_MAX_ENTRIES; i++)
  {
    ResidentChunk* e = &r->entries[i];
    if (e->used && e->buffer == buffer)
    {
      if (e->pins) e->pins--;
      break;
    }
  }
  pthread_mutex_unlock(&r->lock);
}

uint64_t cqlops_resident_evict(CqlResident* r, uint64_t bytes_wanted)
{
  return r ? evict(r, bytes_wanted) : 0;
}

void cqlops_resident_clear(CqlResident* r)
{
  if (!r) return;
  for (;;)
  {
    Doomed d = { { 0 }, 0 };
    pthread_mutex_lock(&r->lock);
    for (int i = 0; i < RESIDENT_MAX_ENTRIES && d.n < 64; i++)
      if (r->entries[i].used && r->entries[i].pins == 0 && r->entries[i].ready) unlink_entry(r, &r->entries[i], &d);
    pthread_mutex_unlock(&r->lock);
    uint32_t n = d.n;
    doom_release(r, &d);
    if (n < 64) return;
  }
}

CqlResidentStats cqlops_resident_stats(CqlResident* r)
{
  CqlResidentStats s;
  memset(&s, 0, sizeof(s));
  if (!r) return s;
  uint64_t b = budget(r);
  pthread_mutex_lock(&r->lock);
  s.hit_bytes = r->hit_bytes;
  s.miss_bytes = r->miss_bytes;
  s.evicted_bytes = r->evicted_bytes;
  s.bytes_in_use = r->bytes_in_use;
  s.entries = r->entry_count;
  s.budget_bytes = b;
  pthread_mutex_unlock(&r->lock);
  return s;
}

static int refuse(const char* why)
{
  cqlops_note_error(why);
  return 0;
}

/* ---- a streamed operator over the cache ----
   SUM/MIN/MAX of a host column in chunks through the cache (qe_aggregate_global_streamed,
   src/query_exec/query_exec.c:8842-9112): each chunk's device copy comes from the cache, or is uploaded
   into it, and cqlops_aggregate_global reduces it; the chunks' partials are folded in chunk order. A
   column larger than device memory passes through the cache's budget chunk by chunk, and a column
   queried again is read from HBM without an upload. */
int cqlops_aggregate_global_streamed(CqlResident* r, uint64_t column_uid, uint64_t generation, const void* host_values, uint32_t type,
                                     uint64_t rows, uint64_t chunk_rows, double* out_sum, double* out_min, double* out_max,
                                     uint64_t* out_uploaded_bytes)
{
  cqlops_note_error("");
  if (out_uploaded_bytes) *out_uploaded_bytes = 0;
  if (!r || r->ops.alloc != dev_alloc) return refuse("the streamed aggregate takes a cache of backend buffers (created with ops NULL)");
  uint32_t width = type == CQLOPS_TYPE_F64 ? 8 : (type == CQLOPS_TYPE_U32 || type == CQLOPS_TYPE_I32 || type == CQLOPS_TYPE_F32) ? 4 : 0;
  if (!width || !host_values || !out_sum || !out_min || !out_max) return refuse("a U32/I32/F32/F64 host column and its outputs");
  if (chunk_rows == 0) chunk_rows = 1u << 24;
  /* one running total over every workgroup partial of every chunk (qe_agg_stream_begin / _retire) */
  double sum = 0.0, mn = 1.7976931348623157e308, mx = -1.7976931348623157e308;
  for (uint64_t start = 0; start < rows; start += chunk_rows)
  {
    uint64_t n = rows - start < chunk_rows ? rows - start : chunk_rows;
    int hit = 0;
    CqlBuffer* b = (CqlBuffer*)cqlops_resident_acquire(r, column_uid, generation, (const char*)host_values + start * width, start, n, width, &hit);
    if (!b) return refuse("a chunk could not be held in the cache");
    if (!hit && out_uploaded_bytes) *out_uploaded_bytes += n * width;
    CqlColumn col;
    memset(&col, 0, sizeof(col));
    col.type = type;
    col.rows = n;
    col.buffer = b;
    int ok = cqlops_aggregate_global_accumulate(&col, 1, &sum, &mn, &mx);
    cqlops_resident_release(r, b);
    if (!ok) return 0;
  }
  *out_sum = sum;
  *out_min = mn;
  *out_max = mx;
  return 1;
}

/* ---- streamed scan and dense group-by over the cache ---- */

static uint32_t host_width(uint32_t type)
{
  return type == CQLOPS_TYPE_F64 ? 8u : (type == CQLOPS_TYPE_U32 || type == CQLOPS_TYPE_I32 || type == CQLOPS_TYPE_F32) ? 4u : 0u;
}

/* a chunk of a host column as a device column: from the cache, or uploaded into it */
static int chunk_column(CqlResident* r, const CqlHostColumn* h, uint64_t start, uint64_t n, CqlColumn* out, uint64_t* uploaded)
{
  uint32_t width = host_width(h->type);
  if (!width || !h->values) return refuse("streamed columns are U32, I32, F32 or F64 host columns");
  int hit = 0;
  CqlBuffer* b = (CqlBuffer*)cqlops_resident_acquire(r, h->uid, h->generation, (const char*)h->values + start * width, start, n, width, &hit);
  if (!b) return refuse("a chunk could not be held in the cache");
  if (!hit && uploaded) *uploaded += n * width;
  memset(out, 0, sizeof(*out));
  out->type = h->type;
  out->rows = n;
  out->buffer = b;
  out->has_range = h->has_range;
  out->zone_min = h->zone_min;
  out->zone_max = h->zone_max;
  return 1;
}

int cqlops_scan_simple_streamed(CqlResident* r, const CqlHostColumn* columns, uint32_t column_count, uint64_t rows, const CqlLeaf* leaves,
                                uint32_t leaf_count, uint64_t chunk_rows, uint64_t* out_count, uint32_t* out_rows, uint64_t out_capacity,
                                uint64_t* out_uploaded_bytes)
{
  cqlops_note_error("");
  if (out_uploaded_bytes) *out_uploaded_bytes = 0;
  if (!r || r->ops.alloc != dev_alloc) return refuse("the streamed scan takes a cache of backend buffers (created with ops NULL)");
  if (!columns || column_count == 0 || column_count > CQLOPS_MAX_BINDINGS || !out_count) return refuse("1 to 10 columns and a count");
  if (!cqlops_rows_fit(rows)) return 0;
  if (chunk_rows == 0) chunk_rows = 1u << 24;
  uint64_t total = 0;
  for (uint64_t start = 0; start < rows; start += chunk_rows)
  {
    uint64_t n = rows - start < chunk_rows ? rows - start : chunk_rows;
    CqlColumn cols[CQLOPS_MAX_BINDINGS];
    uint32_t held = 0;
    int ok = 1;
    for (uint32_t c = 0; c < column_count && ok; c++)
    {
      ok = chunk_column(r, &columns[c], start, n, &cols[c], out_uploaded_bytes);
      if (ok) held++;
    }
    uint64_t got = 0;
    uint64_t room = out_rows && out_capacity > total ? out_capacity - total : 0;
    if (ok) ok = cqlops_scan_simple(cols, column_count, leaves, leaf_count, &got, room ? out_rows + total : NULL, room);
    for (uint32_t c = 0; c < held; c++) cqlops_resident_release(r, cols[c].buffer);
    if (!ok) return 0;
    /* the chunk's rows are its own: offset by its first row */
    uint64_t kept = got < room ? got : room;
    for (uint64_t i = 0; i < kept; i++) out_rows[total + i] += (uint32_t)start;
    total += got;
  }
  *out_count = total;
  return 1;
}

int cqlops_group_dense_streamed(CqlResident* r, const CqlHostColumn* key, uint64_t rows, uint32_t expr_count, const uint32_t* funcs,
                                const CqlHostColumn* const* args, uint64_t chunk_rows, uint64_t max_groups, uint64_t* out_group_count,
                                int64_t* out_min_key, uint64_t* out_counts, int64_t* out_sums, int64_t* out_mins, int64_t* out_maxs,
                                uint64_t* out_uploaded_bytes)
{
  cqlops_note_error("");
  if (out_uploaded_bytes) *out_uploaded_bytes = 0;
  if (!r || r->ops.alloc != dev_alloc) return refuse("the streamed group-by takes a cache of backend buffers (created with ops NULL)");
  if (!key || !key->has_range || expr_count == 0 || expr_count > 8) return refuse("a key with its range and 1 to 8 aggregates");
  if (!out_group_count || !out_min_key || !out_counts || !out_sums || !out_mins || !out_maxs) return refuse("every output array is required");
  if (!cqlops_rows_fit(rows)) return 0;
  if (chunk_rows == 0) chunk_rows = 1u << 24;
  uint64_t groups = (uint64_t)(key->zone_max - key->zone_min) + 1;
  if (groups > max_groups) return refuse("the output arrays hold fewer groups than the key's range");
  uint64_t* c_counts = (uint64_t*)malloc(groups * 8);
  int64_t* c_sums = (int64_t*)malloc(groups * expr_count * 8);
  int64_t* c_mins = (int64_t*)malloc(groups * expr_count * 8);
  int64_t* c_maxs = (int64_t*)malloc(groups * expr_count * 8);
  int ok = c_counts && c_sums && c_mins && c_maxs;
  int first = 1;
  uint64_t g_count = 0;
  int64_t min_key = 0;
  for (uint64_t start = 0; ok && start < rows; start += chunk_rows)
  {
    uint64_t n = rows - start < chunk_rows ? rows - start : chunk_rows;
    CqlColumn kc, ac[8];
    const CqlColumn* argp[8] = { NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL };
    CqlBuffer* held[9];
    uint32_t nheld = 0;
    ok = chunk_column(r, key, start, n, &kc, out_uploaded_bytes);
    if (ok) held[nheld++] = kc.buffer;
    for (uint32_t e = 0; ok && e < expr_count; e++)
    {
      if (!args || !args[e] || funcs[e] == CQLOPS_FUNC_COUNT) continue;
      if (args[e] == key)
      {
        argp[e] = &kc;
        continue;
      }
      uint32_t same = e;
      for (uint32_t j = 0; j < e; j++)
        if (args && args[j] == args[e] && argp[j]) same = j;
      if (same != e)
      {
        argp[e] = argp[same];
        continue;
      }
      ok = chunk_column(r, args[e], start, n, &ac[e], out_uploaded_bytes);
      if (ok)
      {
        held[nheld++] = ac[e].buffer;
        argp[e] = &ac[e];
      }
    }
    /* the first chunk writes straight into the outputs, later chunks into the chunk arrays, folded after */
    uint64_t gc = 0;
    int64_t mk = 0;
    if (ok)
      ok = first ? cqlops_group_dense(&kc, n, expr_count, funcs, argp, max_groups, &gc, &mk, out_counts, out_sums, out_mins, out_maxs)
                 : cqlops_group_dense(&kc, n, expr_count, funcs, argp, groups, &gc, &mk, c_counts, c_sums, c_mins, c_maxs);
    for (uint32_t i = 0; i < nheld; i++) cqlops_resident_release(r, held[i]);
    if (!ok) break;
    if (first)
    {
      g_count = gc;
      min_key = mk;
      first = 0;
      continue;
    }
    if (gc != g_count || mk != min_key)
    {
      ok = refuse("a chunk's groups did not line up with the key's range");
      break;
    }
    for (uint64_t g = 0; g < gc; g++)
    {
      out_counts[g] += c_counts[g];
      for (uint32_t e = 0; e < expr_count; e++)
      {
        uint64_t i = g * expr_count + e;
        out_sums[i] += c_sums[i];
        if (c_mins[i] < out_mins[i]) out_mins[i] = c_mins[i];
        if (c_maxs[i] > out_maxs[i]) out_maxs[i] = c_maxs[i];
      }
    }
  }
  free(c_counts);
  free(c_sums);
  free(c_mins);
  free(c_maxs);
  if (!ok) return 0;
  if (first)
  {
    /* no rows: the groups of the key's range, all empty */
    g_count = groups;
    min_key = (int64_t)key->zone_min;
    for (uint64_t g = 0; g < groups; g++)
    {
      out_counts[g] = 0;
      for (uint32_t e = 0; e < expr_count; e++)
      {
        out_sums[g * expr_count + e] = 0;
        out_mins[g * expr_count + e] = INT32_MAX;
        out_maxs[g * expr_count + e] = INT32_MIN;
      }
    }
  }
  *out_group_count = g_count;
  *out_min_key = min_key;
  return 1;
}
