/*
 * oracle_join.c - join-aggregate over a fact key column and a dimension (TEST INFRASTRUCTURE ONLY).
 *
 * SELECT g, COUNT(*), SUM(arg) FROM fact JOIN dim ON fact.key = dim.k [WHERE <dim rows kept>] GROUP BY g,
 * the result qe_aggregate_join_pushdown (src/query_exec/query_exec.c:8442-8815) returns: the kept
 * dimension rows go into a linear-probing table of their keys, each fact row probes it, and a hit
 * adds the row to its dimension row's group. Integer sums are exact (64-bit). Fact rows are split
 * into ranges over the host threads; each range keeps its own per-group totals, merged at the end.
 */
#include "oracle.h"

#include <stdlib.h>

typedef struct
{
  const uint32_t* fact_key;
  const uint32_t* fact_arg;
  uint64_t rows;
  uint64_t per;
  const uint32_t* table_key;
  const uint32_t* table_group;
  uint64_t mask;
  uint32_t groups;
  uint64_t* counts;  /* [task][groups] */
  int64_t* sums;     /* [task][groups] */
} join_ctx;

static uint64_t join_hash(uint32_t k)
{
  uint64_t h = (uint64_t)k * 0x9E3779B97F4A7C15ull;
  return h ^ (h >> 29);
}

static void orc_join_task(void* p, uint32_t id)
{
  join_ctx* c = (join_ctx*)p;
  uint64_t lo = (uint64_t)id * c->per, hi = lo + c->per < c->rows ? lo + c->per : c->rows;
  uint64_t* cnt = c->counts + (uint64_t)id * c->groups;
  int64_t* sum = c->sums + (uint64_t)id * c->groups;
  for (uint64_t r = lo; r < hi; r++)
  {
    uint32_t k = c->fact_key[r];
    uint64_t s = join_hash(k) & c->mask;
    while (c->table_group[s] != 0xffffffffu)
    {
      if (c->table_key[s] == k)
      {
        uint32_t g = c->table_group[s];
        cnt[g] += 1;
        if (c->fact_arg) sum[g] += c->fact_arg[r];
        break;
      }
      s = (s + 1) & c->mask;
    }
  }
}

void orc_parallel_for(uint32_t tasks, void (*fn)(void*, uint32_t), void* ctx);

int orc_join_aggregate(const uint32_t* fact_key, const uint32_t* fact_arg, uint64_t rows, const uint32_t* dim_key,
                       const uint32_t* dim_group, uint64_t dim_count, uint32_t groups, uint64_t* out_counts, int64_t* out_sums)
{
  uint64_t size = 16;
  while (size < dim_count * 2) size <<= 1;
  uint32_t* tk = (uint32_t*)malloc(size * sizeof(uint32_t));
  uint32_t* tg = (uint32_t*)malloc(size * sizeof(uint32_t));
  if (!tk || !tg) return 0;
  for (uint64_t i = 0; i < size; i++) tg[i] = 0xffffffffu;
  for (uint64_t d = 0; d < dim_count; d++)
  {
    if (dim_group[d] == 0xffffffffu) continue;   /* filtered out */
    uint64_t s = join_hash(dim_key[d]) & (size - 1);
    while (tg[s] != 0xffffffffu) s = (s + 1) & (size - 1);
    tk[s] = dim_key[d];
    tg[s] = dim_group[d];
  }
  uint32_t tasks = orc_threads();
  if (rows < 65536) tasks = 1;
  join_ctx c = { fact_key, fact_arg, rows, (rows + tasks - 1) / tasks, tk, tg, size - 1, groups, NULL, NULL };
  c.counts = (uint64_t*)calloc((uint64_t)tasks * groups, sizeof(uint64_t));
  c.sums = (int64_t*)calloc((uint64_t)tasks * groups, sizeof(int64_t));
  if (!c.counts || !c.sums) return 0;
  orc_parallel_for(tasks, orc_join_task, &c);
  for (uint32_t g = 0; g < groups; g++)
  {
    out_counts[g] = 0;
    out_sums[g] = 0;
    for (uint32_t t = 0; t < tasks; t++)
    {
      out_counts[g] += c.counts[(uint64_t)t * groups + g];
      out_sums[g] += c.sums[(uint64_t)t * groups + g];
    }
  }
  free(c.counts);
  free(c.sums);
  free(tk);
  free(tg);
  return 1;
}
