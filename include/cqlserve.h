/*
 * cqlserve.h - the served form of the GB300 operators: many client threads' queries over tables resident
 * in HBM, run concurrently instead of one at a time.
 *
 * The reference serves each Postgres-wire connection on its own thread (pg_connection_thread_proc,
 * src/server/pg_server.c:643-760; server_run_pg :762-786) and runs one query at a time under
 * g_query_exec_mutex (src/application.h:34, taken in pg_handle_simple_query :200-253). This server keeps
 * the same request/response shape - a client submits a query and waits for its result - and replaces the
 * process-wide mutex with:
 *
 *   - worker threads, each running its requests on a backend lane of its own (its own CUDA stream,
 *     batch and pooled scratch), so independent queries overlap on the GPU;
 *   - admission by planned device footprint: a request starts only while the planned bytes of the
 *     requests running stay within the memory budget (first come, first served; one larger than the
 *     whole budget fails);
 *   - continuous batching: a free worker takes every filter/aggregate request queued on the same table
 *     (up to max_fuse) and answers them with one shared scan (cqlops_batch_filter_aggregate_cat), so
 *     under load the table is read once per batch rather than once per query; a whole-column aggregate
 *     or group-by takes the identical requests queued behind it and answers them with one run. Requests
 *     that arrive while a scan runs form the next batch.
 *
 * Results do not depend on what a request was batched with: counts are exact and the shared scan's sums
 * are exact sums of scaled integers, independent of order and of the other queries.
 */
#ifndef CQLSERVE_H
#define CQLSERVE_H

#include <stdint.h>

#include "cqlops.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CqlServer CqlServer;

typedef struct CqlServeConfig
{
  uint32_t workers;          /* worker threads, each on its own lane; 0 = 2 */
  uint32_t fuse;             /* 1: filter/aggregate requests queued on one table run in one shared scan, and
                                identical queued requests are answered by one run */
  uint32_t max_fuse;         /* most requests in one shared scan; 0 = 1024 */
  uint32_t rows_per_thread;  /* of the shared scan (4, 8 or 16); 0 = 8 */
  uint64_t memory_budget;    /* planned device bytes the running requests may hold together; 0 = 160 GB,
                                at most 90% of the device memory free at creation */
} CqlServeConfig;

enum
{
  CQLSERVE_FILTER_AGG = 1,   /* SELECT COUNT(*)[, SUM(col)] WHERE <program> */
  CQLSERVE_AGG_GLOBAL = 2,   /* SUM/MIN/MAX of up to 4 whole columns */
  CQLSERVE_GROUP_DENSE = 3,  /* GROUP BY one small-range key with COUNT/SUM/MIN/MAX (cqlops_group_dense) */
  CQLSERVE_CALL = 4,         /* any other operator call: call(ctx) on a worker's lane, 1 = success */
};

typedef int (*CqlServeCall)(void* ctx);

typedef struct CqlServeRequest
{
  /* what to run */
  uint32_t kind;
  uint32_t table;                 /* cqlserve_add_table's index */
  const CqlProgram* program;      /* FILTER_AGG: the WHERE, built over the table's columns */
  int32_t sum_column;             /* FILTER_AGG: the summed column, -1 for COUNT(*) alone */
  uint32_t column_count;          /* AGG_GLOBAL: columns[0..column_count); GROUP_DENSE: columns[0] is the key */
  uint32_t columns[4];
  uint32_t expr_count;            /* GROUP_DENSE: funcs[e] over column args[e] (-1 for COUNT) */
  uint32_t funcs[8];
  int32_t args[8];
  uint64_t max_groups;            /* GROUP_DENSE outputs, caller-owned, as cqlops_group_dense writes them */
  uint64_t* out_counts;
  int64_t* out_sums;
  int64_t* out_mins;
  int64_t* out_maxs;
  CqlServeCall call;              /* CALL */
  void* ctx;
  uint64_t footprint;             /* planned device bytes while it runs; 0 = the server's estimate */
  /* results */
  uint64_t count;                 /* FILTER_AGG: matching rows; GROUP_DENSE: groups */
  int64_t min_key;                /* GROUP_DENSE */
  double sum[4];                  /* FILTER_AGG: sum[0]; AGG_GLOBAL: per column */
  double min[4];
  double max[4];
  int32_t status;                 /* 0 queued or running, 1 done, -1 failed (error says why) */
  uint32_t fused;                 /* requests answered by the run that answered this one: a shared scan, or
                                     identical requests merged (1: alone) */
  uint64_t submit_ns;             /* CLOCK_MONOTONIC: submitted, started, finished */
  uint64_t start_ns;
  uint64_t done_ns;
  char error[128];
  struct CqlServeRequest* next;   /* the server's queue link */
} CqlServeRequest;

typedef struct CqlServeStats
{
  uint64_t submitted, completed, failed;
  uint64_t scans;                 /* shared scans run */
  uint64_t fused_requests;        /* requests answered by shared scans */
  uint64_t max_fused;             /* the largest shared scan */
  uint64_t in_flight_bytes;       /* planned bytes of the requests running now */
  uint64_t peak_in_flight_bytes;
  uint64_t memory_budget;
  uint64_t admission_waits;       /* times the head request waited for memory */
  uint64_t merged_requests;       /* requests answered by an identical request's run */
} CqlServeStats;

/* Starts the workers; NULL when a worker's lane cannot be opened (cqlcuda_last_error says why). */
CqlServer* cqlserve_create(const CqlServeConfig* config);
/* Finishes the queued requests, stops the workers and closes their lanes. */
void cqlserve_destroy(CqlServer* server);
/* Registers a resident table (the columns and their buffers stay valid while the server lives);
   returns its index, or -1. */
int cqlserve_add_table(CqlServer* server, const CqlColumn* columns, uint32_t column_count);
/* Compiles the shared-scan kernel for these WHERE shapes on the table ahead of the first request (the
   literals do not matter: a shape is a query with its literals taken out). */
int cqlserve_prepare(CqlServer* server, uint32_t table, const CqlProgram* const* programs, uint32_t count, const int32_t* sum_columns);
/* Queues a request (status 0); the request must stay valid until it is done. Returns 0 when the
   server is stopping or the request is malformed (status -1, error set). */
int cqlserve_submit(CqlServer* server, CqlServeRequest* request);
/* Waits for the request: 1 when it is done or failed, 0 when timeout_ms passed first (0 = no limit). */
int cqlserve_wait(CqlServer* server, CqlServeRequest* request, uint32_t timeout_ms);
/* Waits until nothing is queued or running. */
void cqlserve_drain(CqlServer* server);
CqlServeStats cqlserve_stats(CqlServer* server);

/* Ready-made CALL requests for the join and ORDER BY templates of a served mix: set request.call to the
   function and request.ctx to its struct; they run on the worker's own lane with no callback into the
   caller's runtime. */
typedef struct CqlServeJoin
{
  CqlJoinAgg query;               /* cqlops_join_aggregate's query (its arrays stay valid while it runs) */
  uint64_t max_groups;
  uint64_t* out_group_dim_row;    /* max_groups entries */
  double* out_results;            /* max_groups x query.expr_count */
  uint64_t groups;                /* out */
  uint32_t strategy;              /* out */
} CqlServeJoin;
int cqlserve_join_call(void* join);

/* SELECT ... WHERE <an AND of comparisons> ORDER BY columns[sort_column] [DESC] LIMIT limit: the WHERE by
   cqlops_scan_simple (up to max_rows matching rows, else the request fails), the kept rows sorted on the
   device (cqlops_sort_rows over them as a selection), the first `limit` row numbers written. */
typedef struct CqlServeSort
{
  const CqlColumn* columns;
  uint32_t column_count;
  const CqlLeaf* leaves;
  uint32_t leaf_count;
  uint32_t sort_column;
  uint32_t desc;
  uint64_t max_rows;
  uint64_t limit;
  uint32_t* out_rows;             /* limit entries */
  uint64_t count;                 /* out: the rows the WHERE kept */
} CqlServeSort;
int cqlserve_sort_call(void* sort);

#ifdef __cplusplus
}
#endif

#endif /* CQLSERVE_H */
