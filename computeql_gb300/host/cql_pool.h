/*
 * cql_pool.h - the host thread pool of the operator layer (the role of the reference's app_thread_pool
 * / tp_for_parallel, src/thread_pool/thread_pool.h): a parallel-for over task ids for host loops that
 * touch every row of a dimension table or every group.
 */
#ifndef CQL_POOL_H
#define CQL_POOL_H

#include <stdint.h>

typedef void (*cql_task_fn)(void* ctx, uint32_t task);

/* Runs fn(ctx, t) for t in [0, tasks) on the pool's workers and the calling thread; returns when all are done. */
void cql_parallel_for(uint32_t tasks, cql_task_fn fn, void* ctx);

/* Threads a parallel-for uses (the workers plus the caller). */
uint32_t cql_pool_threads(void);

#endif
