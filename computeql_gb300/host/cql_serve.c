/*
 * cql_serve.c - the served form: worker threads on their own backend lanes, admission by planned device
 * footprint, and continuous batching of filter/aggregate requests into shared scans.
 *
 * It takes the place of the reference's one-query-at-a-time serving (g_query_exec_mutex,
 * src/application.h:34, held around each query by pg_handle_simple_query, src/server/pg_server.c:200-253).
 *
 * One queue, first come first served. A free worker looks at the head request:
 *   - if the planned bytes of the requests running plus its own exceed the memory budget, it waits for a
 *     request to finish (a request larger than the whole budget fails at once);
 *   - a filter/aggregate request, with fusing on, takes with it every other filter/aggregate request
 *     queued on the same table (up to max_fuse, within the budget): one shared scan answers them all;
 *   - any other request takes with it the identical requests queued (same operator, table, columns and
 *     functions): one run answers them all, its results copied to each;
 *   - a call request runs alone.
 * The worker runs its work on its own lane, publishes the results and wakes the waiters. Requests that
 * arrive while the scans run queue up and form the next batch.
 */
#define _GNU_SOURCE
#include "cqlserve.h"
#include "cql_ops_internal.h"

#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define SERVE_MAX_WORKERS 16
#define SERVE_MAX_TABLES 64
#define SERVE_DEFAULT_BUDGET (160ull << 30)
#define SERVE_SMALL_FOOTPRINT (1ull << 20)
#define TAKE_REJECTED 0xffffffffu

typedef struct
{
  CqlColumn* columns;
  uint32_t column_count;
  CqlBatchCatalog* catalog;
} ServeTable;

struct CqlServer
{
  CqlServeConfig cfg;
  pthread_mutex_t lock;
  pthread_cond_t work;     /* a request queued, memory freed or stopping */
  pthread_cond_t done;     /* a request finished */
  CqlServeRequest* head;
  CqlServeRequest* tail;
  uint32_t running;        /* requests taken by workers and not yet finished */
  int stopping;
  ServeTable tables[SERVE_MAX_TABLES];
  uint32_t table_count;
  pthread_t threads[SERVE_MAX_WORKERS];
  uint32_t started;
  int lane_failed;
  uint32_t lanes_ready;
  CqlServeStats stats;
};

static uint64_t now_ns(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

static void fail(CqlServeRequest* r, const char* why)
{
  r->status = -1;
  snprintf(r->error, sizeof(r->error), "%s", why && why[0] ? why : "failed");
}

/* the planned device bytes of a request: the scratch its operator allocates while it runs */
static uint64_t footprint(const CqlServeRequest* r)
{
  if (r->footprint) return r->footprint;
  switch (r->kind)
  {
  case CQLSERVE_FILTER_AGG:
    /* the shared scan's per-CTA partials (24 bytes per query per CTA, ~1k CTAs) and per-query
       thresholds; the per-query kernel's partials are smaller */
    return SERVE_SMALL_FOOTPRINT + 32ull * 1024;
  case CQLSERVE_GROUP_DENSE:
    return SERVE_SMALL_FOOTPRINT + r->max_groups * (uint64_t)(r->expr_count + 1) * 8ull * 4ull;
  case CQLSERVE_CALL:
    return 0;
  default:
    return SERVE_SMALL_FOOTPRINT;
  }
}

/* ---- running requests (on the worker's lane, without the server lock) ---- */

static void run_alone(CqlServer* sv, CqlServeRequest* r)
{
  ServeTable* t = &sv->tables[r->table];
  int ok = 0;
  switch (r->kind)
  {
  case CQLSERVE_FILTER_AGG:
  {
    uint32_t agg = r->sum_column >= 0 ? (uint32_t)r->sum_column : 0;
    double cnt = 0, sum[4] = { 0 }, mn[4] = { 0 }, mx[4] = { 0 };
    ok = cqlops_fused_filter_aggregate(r->program, t->columns, &agg, r->sum_column >= 0 ? 1 : 0, &cnt, sum, mn, mx);
    if (ok)
    {
      r->count = (uint64_t)cnt;
      r->sum[0] = r->sum_column >= 0 ? sum[0] : 0.0;
      r->min[0] = mn[0];
      r->max[0] = mx[0];
    }
    break;
  }
  case CQLSERVE_AGG_GLOBAL:
  {
    CqlColumn cols[4];
    for (uint32_t c = 0; c < r->column_count; c++) cols[c] = t->columns[r->columns[c]];
    ok = cqlops_aggregate_global(cols, r->column_count, r->sum, r->min, r->max);
    break;
  }
  case CQLSERVE_GROUP_DENSE:
  {
    const CqlColumn* args[8];
    for (uint32_t e = 0; e < r->expr_count; e++) args[e] = r->args[e] >= 0 ? &t->columns[r->args[e]] : NULL;
    const CqlColumn* key = &t->columns[r->columns[0]];
    uint64_t groups = 0;
    ok = cqlops_group_dense(key, key->rows, r->expr_count, r->funcs, args, r->max_groups, &groups, &r->min_key, r->out_counts, r->out_sums,
                            r->out_mins, r->out_maxs);
    r->count = groups;
    break;
  }
  case CQLSERVE_CALL:
    ok = r->call(r->ctx);
    break;
  }
  r->fused = 1;
  if (ok) r->status = 1;
  else
  {
    const char* why = cqlops_last_error();
    fail(r, why && why[0] ? why : cqlcuda_last_error());
  }
}

static void run_shared(CqlServer* sv, CqlServeRequest** group, uint32_t n)
{
  ServeTable* t = &sv->tables[group[0]->table];
  const CqlProgram** programs = (const CqlProgram**)malloc(n * sizeof(*programs));
  int32_t* sums = (int32_t*)malloc(n * 4);
  uint64_t* counts = (uint64_t*)malloc(n * 8);
  double* sumv = (double*)malloc(n * 8);
  int ok = programs && sums && counts && sumv;
  for (uint32_t i = 0; ok && i < n; i++)
  {
    programs[i] = group[i]->program;
    sums[i] = group[i]->sum_column;
  }
  if (ok)
    ok = cqlops_batch_filter_aggregate_cat(t->catalog, programs, n, t->columns, t->column_count, sums, sv->cfg.rows_per_thread, counts, sumv,
                                           NULL);
  if (ok)
  {
    for (uint32_t i = 0; i < n; i++)
    {
      group[i]->count = counts[i];
      group[i]->sum[0] = sumv[i];
      group[i]->fused = n;
      group[i]->status = 1;
    }
  }
  else
  {
    /* a query the shared scan refuses (strings, too many literals) runs on its own kernel */
    for (uint32_t i = 0; i < n; i++) run_alone(sv, group[i]);
  }
  free(programs);
  free(sums);
  free(counts);
  free(sumv);
}

/* two requests that ask the same thing: one run answers both (filter/aggregate requests are fused
   instead; a call request is never merged) */
static int same_request(const CqlServeRequest* a, const CqlServeRequest* b)
{
  if (a->kind != b->kind || a->table != b->table) return 0;
  if (a->kind == CQLSERVE_AGG_GLOBAL)
    return a->column_count == b->column_count && !memcmp(a->columns, b->columns, a->column_count * sizeof(uint32_t));
  if (a->kind == CQLSERVE_GROUP_DENSE)
    return a->columns[0] == b->columns[0] && a->expr_count == b->expr_count && a->max_groups == b->max_groups &&
           !memcmp(a->funcs, b->funcs, a->expr_count * sizeof(uint32_t)) && !memcmp(a->args, b->args, a->expr_count * sizeof(int32_t));
  return 0;
}

/* the first request's results, copied to the others that asked the same */
static void share_results(CqlServeRequest** group, uint32_t n)
{
  const CqlServeRequest* h = group[0];
  for (uint32_t i = 1; i < n; i++)
  {
    CqlServeRequest* r = group[i];
    r->status = h->status;
    memcpy(r->error, h->error, sizeof(r->error));
    r->count = h->count;
    r->min_key = h->min_key;
    memcpy(r->sum, h->sum, sizeof(r->sum));
    memcpy(r->min, h->min, sizeof(r->min));
    memcpy(r->max, h->max, sizeof(r->max));
    if (h->kind == CQLSERVE_GROUP_DENSE && h->status == 1)
    {
      uint64_t g = h->count, e = h->expr_count;
      memcpy(r->out_counts, h->out_counts, g * sizeof(uint64_t));
      memcpy(r->out_sums, h->out_sums, g * e * sizeof(int64_t));
      memcpy(r->out_mins, h->out_mins, g * e * sizeof(int64_t));
      memcpy(r->out_maxs, h->out_maxs, g * e * sizeof(int64_t));
    }
  }
  for (uint32_t i = 0; i < n; i++) group[i]->fused = n;
}

/* ---- the queue ---- */

static void unlink_request(CqlServer* sv, CqlServeRequest* prev, CqlServeRequest* r)
{
  if (prev) prev->next = r->next;
  else sv->head = r->next;
  if (sv->tail == r) sv->tail = prev;
  r->next = NULL;
}

/* With the lock held: takes the head request (and, fusing, the requests that share its scan) when the
   budget admits it. Returns the count taken, 0 when the head must wait, TAKE_REJECTED when the head can
   never fit (it is failed and removed). */
static uint32_t take(CqlServer* sv, CqlServeRequest** group, uint32_t cap, uint64_t* out_bytes)
{
  CqlServeRequest* h = sv->head;
  uint64_t budget = sv->cfg.memory_budget;
  uint64_t fp = footprint(h);
  if (fp > budget)
  {
    unlink_request(sv, NULL, h);
    fail(h, "the request's planned device memory exceeds the server's budget");
    h->done_ns = now_ns();
    sv->stats.failed++;
    pthread_cond_broadcast(&sv->done);
    return TAKE_REJECTED;
  }
  if (sv->stats.in_flight_bytes + fp > budget)
  {
    sv->stats.admission_waits++;
    return 0;
  }
  unlink_request(sv, NULL, h);
  group[0] = h;
  uint32_t n = 1;
  uint64_t bytes = fp;
  if (sv->cfg.fuse && h->kind != CQLSERVE_CALL)
  {
    /* a filter/aggregate request takes the others queued on its table into one shared scan; any other
       request takes the identical ones queued, which its one run answers */
    CqlServeRequest* prev = NULL;
    CqlServeRequest* r = sv->head;
    while (r && n < cap)
    {
      CqlServeRequest* next = r->next;
      uint64_t f = h->kind == CQLSERVE_FILTER_AGG ? footprint(r) : 0;
      int joins = h->kind == CQLSERVE_FILTER_AGG ? (r->kind == CQLSERVE_FILTER_AGG && r->table == h->table) : same_request(h, r);
      if (joins && sv->stats.in_flight_bytes + bytes + f <= budget)
      {
        unlink_request(sv, prev, r);
        group[n++] = r;
        bytes += f;
      }
      else
        prev = r;
      r = next;
    }
  }
  *out_bytes = bytes;
  return n;
}

static void* worker_main(void* arg)
{
  CqlServer* sv = (CqlServer*)arg;
  char tag[32];
  pthread_mutex_lock(&sv->lock);
  uint32_t id = sv->lanes_ready;
  pthread_mutex_unlock(&sv->lock);
  snprintf(tag, sizeof(tag), "serve%u", id);
  int lane = cqlcuda_thread_lane_begin(tag);
  pthread_mutex_lock(&sv->lock);
  sv->lanes_ready++;
  if (!lane) sv->lane_failed = 1;
  pthread_cond_broadcast(&sv->done);
  pthread_mutex_unlock(&sv->lock);
  if (!lane) return NULL;

  uint32_t cap = sv->cfg.fuse ? sv->cfg.max_fuse : 1;
  CqlServeRequest** group = (CqlServeRequest**)malloc(cap * sizeof(*group));
  pthread_mutex_lock(&sv->lock);
  while (group)
  {
    uint32_t n = 0;
    uint64_t bytes = 0;
    for (;;)
    {
      if (sv->head)
      {
        uint32_t got = take(sv, group, cap, &bytes);
        if (got == TAKE_REJECTED) continue;   /* the head failed admission for good: look again */
        if (got)
        {
          n = got;
          break;
        }
      }
      else if (sv->stopping)
        break;
      pthread_cond_wait(&sv->work, &sv->lock);
    }
    if (!n) break;
    sv->running += n;
    sv->stats.in_flight_bytes += bytes;
    if (sv->stats.in_flight_bytes > sv->stats.peak_in_flight_bytes) sv->stats.peak_in_flight_bytes = sv->stats.in_flight_bytes;
    pthread_mutex_unlock(&sv->lock);

    uint64_t t0 = now_ns();
    for (uint32_t i = 0; i < n; i++) group[i]->start_ns = t0;
    if (group[0]->kind == CQLSERVE_FILTER_AGG && (n > 1 || sv->cfg.fuse)) run_shared(sv, group, n);
    else
    {
      run_alone(sv, group[0]);
      if (n > 1) share_results(group, n);
    }
    uint64_t t1 = now_ns();

    pthread_mutex_lock(&sv->lock);
    for (uint32_t i = 0; i < n; i++)
    {
      group[i]->done_ns = t1;
      if (group[i]->status == 1) sv->stats.completed++;
      else sv->stats.failed++;
    }
    if (sv->cfg.fuse && group[0]->kind == CQLSERVE_FILTER_AGG && group[0]->fused == n)
    {
      sv->stats.scans++;
      sv->stats.fused_requests += n;
      if (n > sv->stats.max_fused) sv->stats.max_fused = n;
    }
    else if (n > 1)
      sv->stats.merged_requests += n - 1;
    sv->running -= n;
    sv->stats.in_flight_bytes -= bytes;
    pthread_cond_broadcast(&sv->done);
    pthread_cond_broadcast(&sv->work);   /* memory freed: a waiting head may now fit */
  }
  pthread_mutex_unlock(&sv->lock);
  free(group);
  cqlcuda_thread_lane_end();
  return NULL;
}

/* ---- the API ---- */

CqlServer* cqlserve_create(const CqlServeConfig* config)
{
  CqlServer* sv = (CqlServer*)calloc(1, sizeof(CqlServer));
  if (!sv) return NULL;
  if (config) sv->cfg = *config;
  if (sv->cfg.workers == 0) sv->cfg.workers = 2;
  if (sv->cfg.workers > SERVE_MAX_WORKERS) sv->cfg.workers = SERVE_MAX_WORKERS;
  if (sv->cfg.max_fuse == 0) sv->cfg.max_fuse = 1024;
  if (sv->cfg.rows_per_thread == 0) sv->cfg.rows_per_thread = 8;
  if (!cqlcuda_init())
  {
    free(sv);
    return NULL;
  }
  uint64_t budget = sv->cfg.memory_budget ? sv->cfg.memory_budget : SERVE_DEFAULT_BUDGET;
  uint64_t free_bytes = cqlcuda_device_free_memory();
  if (free_bytes && budget > free_bytes / 10 * 9) budget = free_bytes / 10 * 9;
  sv->cfg.memory_budget = budget;
  sv->stats.memory_budget = budget;
  pthread_mutex_init(&sv->lock, NULL);
  pthread_cond_init(&sv->work, NULL);
  pthread_condattr_t ca;
  pthread_condattr_init(&ca);
  pthread_condattr_setclock(&ca, CLOCK_MONOTONIC);
  pthread_cond_init(&sv->done, &ca);
  pthread_condattr_destroy(&ca);
  for (uint32_t w = 0; w < sv->cfg.workers; w++)
  {
    pthread_mutex_lock(&sv->lock);
    uint32_t before = sv->lanes_ready;
    pthread_mutex_unlock(&sv->lock);
    if (pthread_create(&sv->threads[w], NULL, worker_main, sv) != 0) break;
    sv->started++;
    /* one at a time, so that each takes the next lane number */
    pthread_mutex_lock(&sv->lock);
    while (sv->lanes_ready == before) pthread_cond_wait(&sv->done, &sv->lock);
    pthread_mutex_unlock(&sv->lock);
  }
  if (sv->started != sv->cfg.workers || sv->lane_failed)
  {
    cqlserve_destroy(sv);
    return NULL;
  }
  return sv;
}

void cqlserve_destroy(CqlServer* sv)
{
  if (!sv) return;
  pthread_mutex_lock(&sv->lock);
  sv->stopping = 1;
  pthread_cond_broadcast(&sv->work);
  pthread_mutex_unlock(&sv->lock);
  for (uint32_t w = 0; w < sv->started; w++) pthread_join(sv->threads[w], NULL);
  for (uint32_t t = 0; t < sv->table_count; t++)
  {
    free(sv->tables[t].columns);
    cqlops_batch_catalog_destroy(sv->tables[t].catalog);
  }
  pthread_cond_destroy(&sv->work);
  pthread_cond_destroy(&sv->done);
  pthread_mutex_destroy(&sv->lock);
  free(sv);
}

int cqlserve_add_table(CqlServer* sv, const CqlColumn* columns, uint32_t column_count)
{
  if (!sv || !columns || column_count == 0 || column_count > CQLOPS_MAX_BINDINGS) return -1;
  pthread_mutex_lock(&sv->lock);
  int index = -1;
  if (sv->table_count < SERVE_MAX_TABLES)
  {
    ServeTable* t = &sv->tables[sv->table_count];
    t->columns = (CqlColumn*)malloc(column_count * sizeof(CqlColumn));
    t->catalog = cqlops_batch_catalog_create();
    if (t->columns && t->catalog)
    {
      memcpy(t->columns, columns, column_count * sizeof(CqlColumn));
      t->column_count = column_count;
      index = (int)sv->table_count++;
    }
    else
    {
      free(t->columns);
      cqlops_batch_catalog_destroy(t->catalog);
      t->columns = NULL;
      t->catalog = NULL;
    }
  }
  pthread_mutex_unlock(&sv->lock);
  return index;
}

int cqlserve_prepare(CqlServer* sv, uint32_t table, const CqlProgram* const* programs, uint32_t count, const int32_t* sum_columns)
{
  if (!sv || table >= sv->table_count) return 0;
  ServeTable* t = &sv->tables[table];
  return cqlops_batch_prepare(t->catalog, programs, count, t->columns, t->column_count, sum_columns, sv->cfg.rows_per_thread);
}

static int well_formed(CqlServer* sv, CqlServeRequest* r, const char** why)
{
  *why = "";
  if (r->kind == CQLSERVE_CALL) return r->call != NULL || ((*why = "a call request needs its function"), 0);
  if (r->table >= sv->table_count) return (*why = "no such table"), 0;
  ServeTable* t = &sv->tables[r->table];
  switch (r->kind)
  {
  case CQLSERVE_FILTER_AGG:
    if (!r->program) return (*why = "a filter request needs its program"), 0;
    if (r->sum_column >= (int32_t)t->column_count) return (*why = "the summed column is not in the table"), 0;
    return 1;
  case CQLSERVE_AGG_GLOBAL:
    if (r->column_count == 0 || r->column_count > 4) return (*why = "1 to 4 columns"), 0;
    for (uint32_t c = 0; c < r->column_count; c++)
      if (r->columns[c] >= t->column_count) return (*why = "a column is not in the table"), 0;
    return 1;
  case CQLSERVE_GROUP_DENSE:
    if (r->columns[0] >= t->column_count || r->expr_count == 0 || r->expr_count > 8) return (*why = "a key and 1 to 8 expressions"), 0;
    for (uint32_t e = 0; e < r->expr_count; e++)
      if (r->args[e] >= (int32_t)t->column_count) return (*why = "an argument is not in the table"), 0;
    if (!r->out_counts || !r->out_sums || !r->out_mins || !r->out_maxs) return (*why = "a group request needs its outputs"), 0;
    return 1;
  default:
    return (*why = "unknown request kind"), 0;
  }
}

int cqlserve_submit(CqlServer* sv, CqlServeRequest* r)
{
  if (!sv || !r) return 0;
  r->status = 0;
  r->fused = 0;
  r->error[0] = 0;
  r->next = NULL;
  r->submit_ns = now_ns();
  r->start_ns = r->done_ns = 0;
  const char* why;
  pthread_mutex_lock(&sv->lock);
  sv->stats.submitted++;
  if (sv->stopping || !well_formed(sv, r, &why))
  {
    fail(r, sv->stopping ? "the server is stopping" : why);
    r->done_ns = r->submit_ns;
    sv->stats.failed++;
    pthread_mutex_unlock(&sv->lock);
    return 0;
  }
  if (sv->tail) sv->tail->next = r;
  else sv->head = r;
  sv->tail = r;
  pthread_cond_signal(&sv->work);
  pthread_mutex_unlock(&sv->lock);
  return 1;
}

int cqlserve_wait(CqlServer* sv, CqlServeRequest* r, uint32_t timeout_ms)
{
  if (!sv || !r) return 0;
  struct timespec until;
  clock_gettime(CLOCK_MONOTONIC, &until);
  until.tv_sec += timeout_ms / 1000;
  until.tv_nsec += (long)(timeout_ms % 1000) * 1000000L;
  if (until.tv_nsec >= 1000000000L)
  {
    until.tv_sec += 1;
    until.tv_nsec -= 1000000000L;
  }
  pthread_mutex_lock(&sv->lock);
  int finished = 1;
  while (r->status == 0)
  {
    if (timeout_ms == 0) pthread_cond_wait(&sv->done, &sv->lock);
    else if (pthread_cond_timedwait(&sv->done, &sv->lock, &until) != 0 && r->status == 0)
    {
      finished = 0;
      break;
    }
  }
  pthread_mutex_unlock(&sv->lock);
  return finished;
}

void cqlserve_drain(CqlServer* sv)
{
  if (!sv) return;
  pthread_mutex_lock(&sv->lock);
  while (sv->head || sv->running) pthread_cond_wait(&sv->done, &sv->lock);
  pthread_mutex_unlock(&sv->lock);
}

CqlServeStats cqlserve_stats(CqlServer* sv)
{
  CqlServeStats s;
  memset(&s, 0, sizeof(s));
  if (!sv) return s;
  pthread_mutex_lock(&sv->lock);
  s = sv->stats;
  pthread_mutex_unlock(&sv->lock);
  return s;
}

/* ---- ready-made call requests ---- */

int cqlserve_join_call(void* ctx)
{
  CqlServeJoin* j = (CqlServeJoin*)ctx;
  if (!j) return 0;
  return cqlops_join_aggregate(&j->query, j->max_groups, &j->groups, j->out_group_dim_row, j->out_results, &j->strategy);
}

int cqlserve_sort_call(void* ctx)
{
  CqlServeSort* q = (CqlServeSort*)ctx;
  if (!q || !q->columns || q->sort_column >= q->column_count || !q->out_rows) return 0;
  uint64_t cap = q->max_rows ? q->max_rows : 1;
  uint32_t* rows = (uint32_t*)malloc(cap * 4);
  uint32_t* sorted = (uint32_t*)malloc(cap * 4);
  uint64_t n = 0;
  int ok = rows && sorted && cqlops_scan_simple(q->columns, q->column_count, q->leaves, q->leaf_count, &n, rows, cap);
  if (ok && n > cap)
  {
    cqlops_note_error("ORDER BY: more rows passed the WHERE than max_rows");
    ok = 0;
  }
  q->count = ok ? n : 0;
  if (ok && n > 0)
  {
    /* the kept rows as a device selection (a pooled buffer of the worker's lane), sorted there */
    CqlBuffer* sel = cqlcuda_buffer_alloc_pooled("serve_sort_rows", 15, n * 4, CQLCUDA_BUFFER_WRITE, NULL);
    ok = sel != NULL;
    if (ok)
    {
      CqlBatch* b = cqlcuda_batch_begin(n * 4, 0);
      cqlcuda_batch_buffer_write(b, sel, rows, n * 4);
      ok = cqlcuda_batch_end(b);
    }
    ok = ok && cqlops_sort_rows(&q->columns[q->sort_column], 1, &q->desc, sel, n, sorted, n);
    uint64_t k = q->limit < n ? q->limit : n;
    if (ok) memcpy(q->out_rows, sorted, k * 4);
  }
  free(rows);
  free(sorted);
  return ok;
}
