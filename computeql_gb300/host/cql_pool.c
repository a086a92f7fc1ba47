/*
 * cql_pool.c - a persistent pool of host worker threads for the operator layer's host loops.
 *
 * Workers start on first use (one per online core beyond the caller, at most 63) and sleep on a
 * condition variable between jobs. A job hands out task ids from one 64-bit counter holding the job's
 * generation in its high half, taken by compare-and-swap, so a worker that wakes late for a finished
 * job can never take an id of the next one. The caller works too and waits for the last task. One job
 * runs at a time. A process forked after the workers started gets a fresh pool.
 */
#define _GNU_SOURCE
#include "cql_pool.h"

#include <pthread.h>
#include <stdlib.h>
#include <unistd.h>

#define CQL_POOL_MAX_WORKERS 63

typedef struct
{
  pthread_mutex_t lock;
  pthread_cond_t wake;
  pthread_cond_t done;
  pthread_mutex_t job_lock;
  uint32_t workers;
  pid_t pid;
  uint32_t generation;
  cql_task_fn fn;
  void* ctx;
  uint32_t tasks;
  uint64_t counter;    /* generation << 32 | next task id (atomic) */
  uint32_t finished;   /* tasks of the current job finished (atomic) */
  uint32_t started;
} CqlPool;

static CqlPool g_pool = { PTHREAD_MUTEX_INITIALIZER, PTHREAD_COND_INITIALIZER, PTHREAD_COND_INITIALIZER, PTHREAD_MUTEX_INITIALIZER,
                          0, 0, 0, NULL, NULL, 0, 0, 0, 0 };

static void run_tasks(CqlPool* p, uint32_t generation, cql_task_fn fn, void* ctx, uint32_t tasks)
{
  for (;;)
  {
    uint64_t c = __atomic_load_n(&p->counter, __ATOMIC_ACQUIRE);
    if ((uint32_t)(c >> 32) != generation || (uint32_t)c >= tasks) break;
    if (!__atomic_compare_exchange_n(&p->counter, &c, c + 1, 0, __ATOMIC_ACQ_REL, __ATOMIC_ACQUIRE)) continue;
    fn(ctx, (uint32_t)c);
    if (__atomic_add_fetch(&p->finished, 1u, __ATOMIC_ACQ_REL) == tasks)
    {
      pthread_mutex_lock(&p->lock);
      pthread_cond_broadcast(&p->done);
      pthread_mutex_unlock(&p->lock);
    }
  }
}

static void* worker_main(void* arg)
{
  CqlPool* p = (CqlPool*)arg;
  uint32_t seen = 0;
  pthread_mutex_lock(&p->lock);
  for (;;)
  {
    while (p->generation == seen) pthread_cond_wait(&p->wake, &p->lock);
    seen = p->generation;
    cql_task_fn fn = p->fn;
    void* ctx = p->ctx;
    uint32_t tasks = p->tasks;
    pthread_mutex_unlock(&p->lock);
    run_tasks(p, seen, fn, ctx, tasks);
    pthread_mutex_lock(&p->lock);
  }
  return NULL;
}

static void pool_start(CqlPool* p)
{
  pid_t me = getpid();
  if (p->started && p->pid == me) return;
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  uint32_t want = n > 1 ? (uint32_t)(n - 1) : 0;
  if (want > CQL_POOL_MAX_WORKERS) want = CQL_POOL_MAX_WORKERS;
  p->workers = 0;
  p->generation = 0;
  pthread_attr_t attr;
  pthread_attr_init(&attr);
  pthread_attr_setdetachstate(&attr, PTHREAD_CREATE_DETACHED);
  for (uint32_t i = 0; i < want; i++)
  {
    pthread_t th;
    if (pthread_create(&th, &attr, worker_main, p) != 0) break;
    p->workers++;
  }
  pthread_attr_destroy(&attr);
  p->pid = me;
  p->started = 1;
}

uint32_t cql_pool_threads(void)
{
  CqlPool* p = &g_pool;
  pthread_mutex_lock(&p->job_lock);
  pthread_mutex_lock(&p->lock);
  pool_start(p);
  uint32_t n = p->workers + 1;
  pthread_mutex_unlock(&p->lock);
  pthread_mutex_unlock(&p->job_lock);
  return n;
}

void cql_parallel_for(uint32_t tasks, cql_task_fn fn, void* ctx)
{
  if (tasks == 0) return;
  CqlPool* p = &g_pool;
  pthread_mutex_lock(&p->job_lock);
  pthread_mutex_lock(&p->lock);
  pool_start(p);
  if (p->workers == 0 || tasks == 1)
  {
    pthread_mutex_unlock(&p->lock);
    for (uint32_t t = 0; t < tasks; t++) fn(ctx, t);
    pthread_mutex_unlock(&p->job_lock);
    return;
  }
  p->fn = fn;
  p->ctx = ctx;
  p->tasks = tasks;
  p->generation++;
  uint32_t generation = p->generation;
  __atomic_store_n(&p->finished, 0u, __ATOMIC_RELEASE);
  __atomic_store_n(&p->counter, (uint64_t)generation << 32, __ATOMIC_RELEASE);
  pthread_cond_broadcast(&p->wake);
  pthread_mutex_unlock(&p->lock);
  run_tasks(p, generation, fn, ctx, tasks);
  pthread_mutex_lock(&p->lock);
  while (__atomic_load_n(&p->finished, __ATOMIC_ACQUIRE) < tasks) pthread_cond_wait(&p->done, &p->lock);
  pthread_mutex_unlock(&p->lock);
  pthread_mutex_unlock(&p->job_lock);
}
