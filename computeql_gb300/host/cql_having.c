/*
 * cql_having.c - a HAVING condition over the grouped result, evaluated for every group at once
 * (qk_having_kernel, src/query_exec/query_kernel.c:2530-2575).
 *
 * The condition is an expression over v0..v7 (the values of the group's result columns, as doubles) and
 * lit[0..15] (its literals), in the C-like syntax the reference's generated GLSL takes. It becomes the
 * body of a generated kernel - one group per thread, keep[i] = 1 when group i passes - compiled by NVRTC
 * and cached by its source, so conditions that differ only in their literals share one kernel. The text is
 * checked first: only those names, numbers, operators and a few math functions may appear.
 */
#include "cqlops.h"
#include "cql_ops_internal.h"

#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define HAVING_MAX_COLUMNS 8
#define HAVING_MAX_LITERALS 16

static int refuse(const char* why)
{
  cqlops_note_error(why);
  return 0;
}

static CqlBuffer* pooled(const char* name, uint64_t size, uint32_t flags)
{
  return cqlcuda_buffer_alloc_pooled(name, (uint64_t)strlen(name), size ? size : 8, flags, NULL);
}

/* 1 when the condition uses only v0..v7, lit[...], numbers, operators, parentheses and the functions
   below; the generated kernel takes nothing else */
static int condition_ok(const char* c, uint32_t column_count)
{
  static const char* const funcs[] = { "fabs", "abs", "fmin", "fmax", "floor", "ceil", "sqrt", "isnan", "true", "false" };
  size_t n = strlen(c);
  if (n == 0 || n > 4096) return 0;
  for (size_t i = 0; i < n;)
  {
    unsigned char ch = (unsigned char)c[i];
    if (isalpha(ch) || ch == '_')
    {
      size_t j = i;
      while (j < n && (isalnum((unsigned char)c[j]) || c[j] == '_')) j++;
      size_t len = j - i;
      int ok = 0;
      if (len == 2 && c[i] == 'v' && c[i + 1] >= '0' && c[i + 1] < '0' + (int)column_count) ok = 1;
      if (len == 3 && !strncmp(c + i, "lit", 3)) ok = 1;
      for (size_t f = 0; !ok && f < sizeof(funcs) / sizeof(funcs[0]); f++) ok = strlen(funcs[f]) == len && !strncmp(c + i, funcs[f], len);
      if (!ok) return 0;
      i = j;
      continue;
    }
    if (isdigit(ch) || ch == '.')
    {
      /* a number: digits, one exponent with its sign */
      size_t j = i;
      while (j < n && (isalnum((unsigned char)c[j]) || c[j] == '.' || ((c[j] == '+' || c[j] == '-') && (c[j - 1] == 'e' || c[j - 1] == 'E'))))
        j++;
      i = j;
      continue;
    }
    if (!strchr(" \t()[]<>=!&|+-*/%,?:", ch)) return 0;
    i++;
  }
  return 1;
}

int cqlops_having_source(const char* condition, uint32_t column_count, char* out, uint64_t cap, uint64_t* out_len)
{
  if (!condition || column_count > HAVING_MAX_COLUMNS) return refuse("HAVING takes up to 8 result columns");
  if (!condition_ok(condition, column_count))
    return refuse("the HAVING condition may use only v0..v7, lit[i], numbers, operators and fabs/fmin/fmax/floor/ceil/sqrt/isnan");
  /* the kernel: one group per thread over a persistent grid; binding 0 keep, 1 literals, 2 + c column c */
  uint64_t need = strlen(condition) + 1024 + 64 * column_count;
  if (cap < need) return refuse("the HAVING source buffer is too small");
  int len = snprintf(out, cap,
                     "// cql: block=256 smem=0 per_sm=8\n"
                     "typedef unsigned int u32;\ntypedef unsigned long long u64;\n"
                     "struct CqlLaunch { void* buf[16]; u64 bytes[16]; u64 push[8]; };\n"
                     "extern \"C\" __global__ void __launch_bounds__(256) cql_main(CqlLaunch a)\n{\n"
                     "  u32* keep = (u32*)a.buf[0]; const double* lit = (const double*)a.buf[1]; (void)lit;\n"
                     "  const u64 n = a.push[0];\n"
                     "  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x)\n  {\n");
  for (uint32_t c = 0; c < column_count; c++)
    len += snprintf(out + len, cap - (uint64_t)len, "    const double v%u = ((const double*)a.buf[%u])[i];\n", c, 2 + c);
  len += snprintf(out + len, cap - (uint64_t)len, "    keep[i] = (%s) ? 1u : 0u;\n  }\n}\n", condition);
  if (out_len) *out_len = (uint64_t)len;
  return 1;
}

int cqlops_having(const char* condition, const double* literals, uint32_t literal_count, const double* const* columns, uint32_t column_count,
                  uint64_t group_count, uint32_t* out_keep)
{
  cqlops_note_error("");
  if (!condition || column_count > HAVING_MAX_COLUMNS || literal_count > HAVING_MAX_LITERALS)
    return refuse("HAVING takes up to 8 result columns and 16 literals");
  if (!condition_ok(condition, column_count))
    return refuse("the HAVING condition may use only v0..v7, lit[i], numbers, operators and fabs/fmin/fmax/floor/ceil/sqrt/isnan");
  if (group_count == 0) return 1;
  if (group_count >= 0xffffffffull) return refuse("too many groups");
  char* src = (char*)malloc(strlen(condition) + 2048);
  if (!src) return 0;
  uint64_t src_len = 0;
  if (!cqlops_having_source(condition, column_count, src, strlen(condition) + 2048, &src_len))
  {
    free(src);
    return 0;
  }
  uint64_t h = 1469598103934665603ull;
  for (const char* p = src; *p; p++) h = (h ^ (unsigned char)*p) * 1099511628211ull;
  char name[48];
  snprintf(name, sizeof(name), "qk_having_%016llx", (unsigned long long)h);
  CqlKernel* k = cqlcuda_kernel_alloc(name, strlen(name));
  if (!k) k = cqlcuda_kernel_alloc_from_image(name, strlen(name), src, strlen(src));
  free(src);
  if (!k) return refuse("the HAVING kernel did not compile");
  CqlBuffer* keep = pooled("having_keep", group_count * 4, CQLCUDA_BUFFER_READ_WRITE);
  CqlBuffer* lit = pooled("having_literals", HAVING_MAX_LITERALS * 8, CQLCUDA_BUFFER_WRITE);
  CqlBuffer* cols[HAVING_MAX_COLUMNS] = { NULL };
  static const char* const col_names[HAVING_MAX_COLUMNS] = { "having_v0", "having_v1", "having_v2", "having_v3",
                                                              "having_v4", "having_v5", "having_v6", "having_v7" };
  int ok = keep && lit;
  for (uint32_t c = 0; ok && c < column_count; c++)
  {
    cols[c] = pooled(col_names[c], group_count * 8, CQLCUDA_BUFFER_WRITE);
    ok = cols[c] != NULL;
  }
  if (!ok) return 0;
  double lits[HAVING_MAX_LITERALS] = { 0 };
  for (uint32_t i = 0; i < literal_count; i++) lits[i] = literals[i];
  cqlcuda_kernel_set_arg_buffer(k, 0, keep);
  cqlcuda_kernel_set_arg_buffer(k, 1, lit);
  for (uint32_t c = 0; c < HAVING_MAX_COLUMNS; c++) cqlcuda_kernel_set_arg_buffer(k, 2 + c, c < column_count ? cols[c] : keep);
  cqlcuda_kernel_set_arg_u64(k, 0, group_count);
  CqlBatch* b = cqlcuda_batch_begin(HAVING_MAX_LITERALS * 8 + group_count * 8 * column_count, group_count * 4);
  cqlcuda_batch_buffer_write(b, lit, lits, sizeof(lits));
  for (uint32_t c = 0; c < column_count; c++) cqlcuda_batch_buffer_write(b, cols[c], columns[c], group_count * 8);
  cqlcuda_batch_kernel_execute(b, k, (uint32_t)(group_count < 0x7fffff00u ? group_count : 0x7fffff00u), 256);
  cqlcuda_batch_buffer_read(b, keep, out_keep, group_count * 4);
  return cqlcuda_batch_end(b);
}
