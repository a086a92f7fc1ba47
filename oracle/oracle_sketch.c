/*
 * oracle_sketch.c - CPU restatement of the reference's HyperLogLog and t-digest (TEST
 * INFRASTRUCTURE ONLY: the checker, never part of the product).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static uint32_t mix32(uint32_t x)
{
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

/* hll_add, src/gpu/vulkan/shaders/aggregate_reduce.comp:66-92 */
void orc_hll_add(const double* values, uint64_t n, uint32_t p, uint32_t* regs)
{
  uint32_t rest_bits = 32u - p;
  for (uint64_t i = 0; i < n; i++)
  {
    uint64_t bits;
    memcpy(&bits, &values[i], sizeof(bits));
    uint32_t h = mix32((uint32_t)bits ^ mix32((uint32_t)(bits >> 32)));
    uint32_t bucket = h >> rest_bits;
    uint32_t rest = h & ((1u << rest_bits) - 1u);
    int msb = -1;
    for (int b = 31; b >= 0; b--)
    {
      if (rest & (1u << b))
      {
        msb = b;
        break;
      }
    }
    uint32_t rho = msb < 0 ? rest_bits + 1u : rest_bits - (uint32_t)msb;
    if (rho > regs[bucket]) regs[bucket] = rho;
  }
}

/* qe_hll_estimate_cardinality, src/query_exec/query_exec.c:6711-6737 */
double orc_hll_estimate(const uint32_t* regs, uint64_t m_count)
{
  double m = (double)m_count;
  double alpha;
  if (m_count == 16) alpha = 0.673;
  else if (m_count == 32) alpha = 0.697;
  else if (m_count == 64) alpha = 0.709;
  else alpha = 0.7213 / (1.0 + 1.079 / m);
  double sum = 0.0;
  uint64_t zeros = 0;
  for (uint64_t i = 0; i < m_count; i++)
  {
    sum += 1.0 / (double)((uint64_t)1 << regs[i]);
    zeros += regs[i] == 0;
  }
  double e = alpha * m * m / sum;
  if (e <= 2.5 * m && zeros > 0) e = m * log(m / (double)zeros);
  return e;
}

typedef struct
{
  float mean, weight;
} OrcCentroid;

static int orc_centroid_cmp(const void* a, const void* b)
{
  float x = ((const OrcCentroid*)a)->mean, y = ((const OrcCentroid*)b)->mean;
  return (x > y) - (x < y);
}

/* qe_tdigest_estimate_percentile, src/query_exec/query_exec.c:6748-6790 */
double orc_tdigest_percentile(float* means, float* weights, uint64_t count, double fraction)
{
  if (count == 0) return 0.0;
  OrcCentroid* c = (OrcCentroid*)malloc(sizeof(OrcCentroid) * count);
  for (uint64_t i = 0; i < count; i++)
  {
    c[i].mean = means[i];
    c[i].weight = weights[i];
  }
  qsort(c, count, sizeof(OrcCentroid), orc_centroid_cmp);
  double total = 0.0;
  for (uint64_t i = 0; i < count; i++) total += c[i].weight;
  double out = (double)c[count - 1].mean;
  if (total <= 0.0) out = 0.0;
  else
  {
    double target = fraction * total, cum = 0.0, prev_pos = -1.0, prev_mean = (double)c[0].mean;
    for (uint64_t i = 0; i < count; i++)
    {
      double pos = cum + (double)c[i].weight * 0.5;
      if (target <= pos)
      {
        out = prev_pos < 0.0 ? (double)c[i].mean : prev_mean + (target - prev_pos) / (pos - prev_pos) * ((double)c[i].mean - prev_mean);
        break;
      }
      cum += c[i].weight;
      prev_pos = pos;
      prev_mean = (double)c[i].mean;
    }
  }
  free(c);
  return out;
}
