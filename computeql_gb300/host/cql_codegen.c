/*
 * cql_codegen.c - per-query CUDA C++ kernels from the scan bytecode.
 *
 * Replaces the GLSL emitter qk_scan_source_build (src/query_exec/query_kernel.c:971-1672): the
 * bytecode is executed symbolically into one boolean expression per row, literals stay in the
 * constant buffer (binding 1) so queries that differ only in literal values share one kernel, and
 * the kernel keeps the binding contract of the kernel it replaces:
 *   CQLOPS_KERNEL_SCAN        scan_filter.comp's bindings: row ids + aux word into binding 3, count
 *                             in binding 4, zone skip bits in binding 5 (query_kernel.c:1616-1670);
 *                             with word 10 set, binding 3 receives a bitmap of the rows instead (each
 *                             32-row word from the four lanes that own it)
 *   CQLOPS_KERNEL_FUSED_AGG   partials [workgroup][1 + 3k] doubles in binding 3 (:1538-1614)
 *   CQLOPS_KERNEL_FUSED_GROUP [group][2 + 4k] words in binding 3 (:1433-1537)
 *
 * GB300 shape of the generated code: each thread evaluates 8 consecutive rows from 16-byte vector
 * loads; matches are compacted with a warp prefix sum of popc() and one global atomic per CTA and
 * pass. A comparison of a whole-number column with a literal becomes an unsigned interval test on
 * the raw word, an F32 column is compared with float bounds, both worked out once per thread from
 * the double literal, so the per-row work stays off the FP64 pipe while the result equals the
 * reference's comparison in double.
 */
#include "cqlops.h"
#include "cql_codegen.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum
{
  OP_PUSH_TRUE = 0, OP_LOAD_NUM_COL = 1, OP_PUSH_CONST = 2, OP_CMP_EQ = 3, OP_CMP_NE = 4, OP_CMP_LT = 5, OP_CMP_GT = 6,
  OP_CMP_LE = 7, OP_CMP_GE = 8, OP_AND = 9, OP_OR = 10, OP_STR_EQ = 11, OP_STR_CONTAINS = 12, OP_HALT = 13, OP_PUSH_FALSE = 14,
  OP_TRIGRAM_SIM = 15, OP_EDIT_DISTANCE = 16, OP_STR_NE = 17, OP_STR_LT = 18, OP_STR_GT = 19, OP_STR_LE = 20, OP_STR_GE = 21,
};

/* ---- a growable string ---- */
typedef struct
{
  char* p;
  size_t n, cap;
  int failed;
} Str;

static void sputs(Str* s, const char* t)
{
  size_t len = strlen(t);
  if (s->n + len + 1 > s->cap)
  {
    size_t cap = s->cap ? s->cap * 2 : 4096;
    while (cap < s->n + len + 1) cap *= 2;
    char* q = (char*)realloc(s->p, cap);
    if (!q)
    {
      s->failed = 1;
      return;
    }
    s->p = q;
    s->cap = cap;
  }
  memcpy(s->p + s->n, t, len + 1);
  s->n += len;
}

static void sprintf_(Str* s, const char* fmt, ...)
{
  char buf[4096];
  va_list ap;
  va_start(ap, fmt);
  int n = vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (n < 0 || n >= (int)sizeof(buf))
  {
    s->failed = 1;
    return;
  }
  sputs(s, buf);
}

/* ---- symbolic values ---- */
typedef struct
{
  char* text;
  int is_bool;
  int col_slot;   /* >= 0: a column load */
  int col_type;
  int const_index; /* >= 0: a literal */
} Val;

static char* dupf(const char* fmt, ...)
{
  char buf[8192];
  va_list ap;
  va_start(ap, fmt);
  int n = vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (n < 0 || n >= (int)sizeof(buf)) return NULL;
  char* p = (char*)malloc((size_t)n + 1);
  if (p) memcpy(p, buf, (size_t)n + 1);
  return p;
}

static int type_bytes(uint32_t t)
{
  switch (t)
  {
    case CQLOPS_TYPE_U32: case CQLOPS_TYPE_F32: case CQLOPS_TYPE_I32: case 9: case 12: return 4;
    case CQLOPS_TYPE_BOOL: return 1;
    case CQLOPS_TYPE_U64: case CQLOPS_TYPE_F64: case CQLOPS_TYPE_I64: case 10: case 11: return 8;
    default: return 0;
  }
}

/* the value of raw row k of a slot widened to double, as read_num_column_value (scan_filter.comp:123-160) */
static char* dbl_of(int slot, int type)
{
  switch (type)
  {
    case CQLOPS_TYPE_U32: case 12: case CQLOPS_TYPE_BOOL: return dupf("((double)r%d[k])", slot);
    case CQLOPS_TYPE_I32: case 9: return dupf("((double)(int)r%d[k])", slot);
    case CQLOPS_TYPE_F32: return dupf("((double)__uint_as_float(r%d[k]))", slot);
    case CQLOPS_TYPE_F64: return dupf("__longlong_as_double((long long)r%d[k])", slot);
    case CQLOPS_TYPE_U64: return dupf("((double)(u32)(r%d[k] >> 32) * 4294967296.0 + (double)(u32)r%d[k])", slot, slot);
    default: return dupf("cql_i64d(r%d[k])", slot);
  }
}

static char* as_double(const Val* v)
{
  if (v->is_bool) return dupf("((%s) ? 1.0 : 0.0)", v->text);
  return dupf("%s", v->text);
}

static char* as_bool(const Val* v)
{
  if (v->is_bool) return dupf("%s", v->text);
  return dupf("((%s) != 0.0)", v->text);
}

typedef struct
{
  const CqlProgram* prog;
  Str pro;       /* per-thread prologue: literals and thresholds */
  int slot_type[CQLOPS_MAX_BINDINGS];  /* type each numeric slot is loaded as, 0 = not loaded */
  int uses_strings;
  int sites;
  int failed;
  char why[128];
  /* batch mode: thresholds and literals come from the query's tables (TH, QC), the sites are listed */
  int batch;
  CqlBatchSite* batch_sites;
  uint32_t batch_cap;
} Gen;

static void gen_fail(Gen* g, const char* why)
{
  if (!g->failed) snprintf(g->why, sizeof(g->why), "%s", why);
  g->failed = 1;
}

static int flip(int op)
{
  switch (op)
  {
    case OP_CMP_LT: return OP_CMP_GT;
    case OP_CMP_GT: return OP_CMP_LT;
    case OP_CMP_LE: return OP_CMP_GE;
    case OP_CMP_GE: return OP_CMP_LE;
    default: return op;
  }
}

static const char* op_text(int op)
{
  switch (op)
  {
    case OP_CMP_EQ: return "==";
    case OP_CMP_NE: return "!=";
    case OP_CMP_LT: return "<";
    case OP_CMP_GT: return ">";
    case OP_CMP_LE: return "<=";
    default: return ">=";
  }
}

/* a comparison of a column with a literal */
static char* column_vs_const(Gen* g, const Val* col, const Val* k, int op)
{
  int site = g->sites++;
  int t = col->col_type;
  if (g->batch)
  {
    if ((uint32_t)site >= g->batch_cap)
    {
      gen_fail(g, "too many comparisons for one batched query");
      return dupf("false");
    }
    CqlBatchSite* bs = &g->batch_sites[site];
    bs->const_index = (uint32_t)k->const_index;
    bs->op = (uint32_t)op;
    bs->col_type = (uint32_t)t;
    bs->pad = 0;
    if (t == CQLOPS_TYPE_U32 || t == 12 || t == CQLOPS_TYPE_BOOL) return dupf("cql_bi(&T%d, r%d[k])", site, col->col_slot);
    if (t == CQLOPS_TYPE_I32 || t == 9) return dupf("cql_bi(&T%d, r%d[k] ^ 0x80000000u)", site, col->col_slot);
    if (t == CQLOPS_TYPE_F32) return dupf("cql_bf(&T%d, __uint_as_float(r%d[k]))", site, col->col_slot);
    if (t == CQLOPS_TYPE_F64) return dupf("cql_bk(&T%d, kd%d[k])", site, col->col_slot);
    gen_fail(g, "a 64-bit integer comparison is not batched");
    return dupf("false");
  }
  if (t == CQLOPS_TYPE_U32 || t == 12 || t == CQLOPS_TYPE_BOOL || t == CQLOPS_TYPE_I32 || t == 9)
  {
    int bias = (t == CQLOPS_TYPE_I32 || t == 9);
    sprintf_(&g->pro, "  const ThrI T%d = cql_thr_int(K%d, %d, %du);\n", site, k->const_index, op, bias ? 1 : 0);
    if (bias) return dupf("T%d.m(r%d[k] ^ 0x80000000u)", site, col->col_slot);
    return dupf("T%d.m(r%d[k])", site, col->col_slot);
  }
  if (t == CQLOPS_TYPE_F32)
  {
    sprintf_(&g->pro, "  const ThrF T%d = cql_thr_f32(K%d, %d);\n", site, k->const_index, op);
    return dupf("T%d.m(__uint_as_float(r%d[k]))", site, col->col_slot);
  }
  if (t == CQLOPS_TYPE_F64)
  {
    /* an interval of order keys of the double: integer work per row, the same answer as comparing in double */
    sprintf_(&g->pro, "  const ThrD T%d = cql_thr_f64(K%d, %d);\n", site, k->const_index, op);
    return dupf("T%d.m(r%d[k])", site, col->col_slot);
  }
  char* d = dbl_of(col->col_slot, t);
  char* r = dupf("(%s %s K%d)", d, op_text(op), k->const_index);
  free(d);
  return r;
}

static void note_slot(Gen* g, int slot, int type)
{
  if (slot < 0 || slot >= CQLOPS_MAX_BINDINGS)
  {
    gen_fail(g, "column slot out of range");
    return;
  }
  if (type_bytes((uint32_t)type) == 0)
  {
    gen_fail(g, "column type without a numeric loader");
    return;
  }
  if (g->slot_type[slot] && g->slot_type[slot] != type)
  {
    gen_fail(g, "one slot read as two types");
    return;
  }
  g->slot_type[slot] = type;
}

/* symbolic execution of the bytecode into one boolean expression over row k */
static char* build_expression(Gen* g)
{
  const CqlProgram* p = g->prog;
  Val stack[64];
  int sp = 0;
  int consts_seen[CQLOPS_MAX_CONSTS] = { 0 };
  uint64_t ip = 0;
  while (!g->failed && ip < p->word_count)
  {
    uint32_t op = p->words[ip++];
    if (op == OP_HALT) break;
    switch (op)
    {
      case OP_PUSH_TRUE:
      case OP_PUSH_FALSE:
        if (sp >= 64) { gen_fail(g, "stack"); break; }
        stack[sp].text = dupf(op == OP_PUSH_TRUE ? "true" : "false");
        stack[sp].is_bool = 1;
        stack[sp].col_slot = -1;
        stack[sp].const_index = -1;
        sp++;
        break;
      case OP_LOAD_NUM_COL:
      {
        if (sp >= 64 || ip >= p->word_count) { gen_fail(g, "stack"); break; }
        uint32_t operand = p->words[ip++];
        int slot = (int)(operand & 0xffu), type = (int)((operand >> 8) & 0xffu);
        note_slot(g, slot, type);
        stack[sp].text = dbl_of(slot, type);
        stack[sp].is_bool = 0;
        stack[sp].col_slot = slot;
        stack[sp].col_type = type;
        stack[sp].const_index = -1;
        sp++;
        break;
      }
      case OP_PUSH_CONST:
      {
        if (sp >= 64 || ip >= p->word_count) { gen_fail(g, "stack"); break; }
        uint32_t index = p->words[ip++];
        if (index >= p->const_count) { gen_fail(g, "constant index"); break; }
        if (!consts_seen[index] && !g->batch)
        {
          consts_seen[index] = 1;
          sprintf_(&g->pro, "  const double K%u = cql_const(a, %uu);\n", index, index);
        }
        stack[sp].text = g->batch ? dupf("QC[%u]", index) : dupf("K%u", index);
        stack[sp].is_bool = 0;
        stack[sp].col_slot = -1;
        stack[sp].const_index = (int)index;
        sp++;
        break;
      }
      case OP_CMP_EQ: case OP_CMP_NE: case OP_CMP_LT: case OP_CMP_GT: case OP_CMP_LE: case OP_CMP_GE:
      {
        if (sp < 2) { gen_fail(g, "stack"); break; }
        Val b = stack[--sp], a = stack[--sp];
        char* r;
        if (!a.is_bool && a.col_slot >= 0 && !b.is_bool && b.const_index >= 0) r = column_vs_const(g, &a, &b, (int)op);
        else if (!b.is_bool && b.col_slot >= 0 && !a.is_bool && a.const_index >= 0) r = column_vs_const(g, &b, &a, flip((int)op));
        else
        {
          char* x = as_double(&a);
          char* y = as_double(&b);
          r = dupf("(%s %s %s)", x, op_text((int)op), y);
          free(x);
          free(y);
        }
        free(a.text);
        free(b.text);
        stack[sp].text = r;
        stack[sp].is_bool = 1;
        stack[sp].col_slot = -1;
        stack[sp].const_index = -1;
        sp++;
        break;
      }
      case OP_AND:
      case OP_OR:
      {
        if (sp < 2) { gen_fail(g, "stack"); break; }
        Val b = stack[--sp], a = stack[--sp];
        char* x = as_bool(&a);
        char* y = as_bool(&b);
        /* numeric-only programs combine without branches; string tests keep the short circuit */
        const char* j = g->uses_strings ? (op == OP_AND ? "&&" : "||") : (op == OP_AND ? "&" : "|");
        char* r = dupf("(%s %s %s)", x, j, y);
        free(x);
        free(y);
        free(a.text);
        free(b.text);
        stack[sp].text = r;
        stack[sp].is_bool = 1;
        stack[sp].col_slot = -1;
        stack[sp].const_index = -1;
        sp++;
        break;
      }
      case OP_STR_EQ: case OP_STR_NE: case OP_STR_LT: case OP_STR_GT: case OP_STR_LE: case OP_STR_GE: case OP_STR_CONTAINS:
      {
        if (g->batch)
        {
          gen_fail(g, "string comparisons are not batched");
          break;
        }
        if (sp >= 64 || ip + 3 > p->word_count) { gen_fail(g, "stack"); break; }
        uint32_t slot = p->words[ip], wo = p->words[ip + 1], len = p->words[ip + 2];
        ip += 3;
        if (slot + 1 >= CQLOPS_MAX_BINDINGS) { gen_fail(g, "string slot"); break; }
        const char* f = op == OP_STR_CONTAINS ? "cql_str_contains(a, %u, row0 + k, %uu, %uu)"
                      : op == OP_STR_EQ ? "cql_str_eq(a, %u, row0 + k, %uu, %uu)"
                      : op == OP_STR_NE ? "!cql_str_eq(a, %u, row0 + k, %uu, %uu)"
                      : op == OP_STR_LT ? "(cql_str_cmp3(a, %u, row0 + k, %uu, %uu) < 0)"
                      : op == OP_STR_GT ? "(cql_str_cmp3(a, %u, row0 + k, %uu, %uu) > 0)"
                      : op == OP_STR_LE ? "(cql_str_cmp3(a, %u, row0 + k, %uu, %uu) <= 0)"
                                        : "(cql_str_cmp3(a, %u, row0 + k, %uu, %uu) >= 0)";
        stack[sp].text = dupf(f, slot, wo, len);
        stack[sp].is_bool = 1;
        stack[sp].col_slot = -1;
        stack[sp].const_index = -1;
        sp++;
        break;
      }
      default:
        gen_fail(g, "an opcode the generated kernel does not take (trigram similarity, edit distance)");
        break;
    }
  }
  char* result = NULL;
  if (!g->failed && sp >= 1) result = as_bool(&stack[sp - 1]);
  else if (!g->failed) gen_fail(g, "empty program");
  for (int i = 0; i < sp; i++) free(stack[i].text);
  return result;
}

static const char* PRELUDE =
  "typedef unsigned int u32;\n"
  "typedef unsigned long long u64;\n"
  "struct CqlLaunch { void* buf[16]; u64 bytes[16]; u64 push[8]; };\n"
  "__device__ __forceinline__ u32 cql_word(const CqlLaunch& a, u32 i) { u64 s = a.push[i >> 1]; return (i & 1u) ? (u32)(s >> 32) : (u32)s; }\n"
  "__device__ __forceinline__ double cql_const(const CqlLaunch& a, u32 k) { const u32* c = (const u32*)a.buf[1]; return __hiloint2double((int)c[2 * k + 1], (int)c[2 * k]); }\n"
  "__device__ __forceinline__ uint4 cql_ld4(const void* p) { uint4 v; asm volatile(\"ld.global.cs.v4.u32 {%0,%1,%2,%3}, [%4];\" : \"=r\"(v.x), \"=r\"(v.y), \"=r\"(v.z), \"=r\"(v.w) : \"l\"(p)); return v; }\n"
  "__device__ __forceinline__ double cql_i64d(u64 x) { double u = (double)(u32)(x >> 32) * 4294967296.0 + (double)(u32)x; return (x >> 63) ? u - 18446744073709551616.0 : u; }\n"
  /* whole-number comparison as an interval of (biased) codes: match = (code - lo <= span) != invert */
  "struct ThrI { u32 lo, span; bool invert; __device__ __forceinline__ bool m(u32 code) const { return ((code - lo) <= span) != invert; } };\n"
  "__device__ ThrI cql_thr_int(double c, int op, u32 biased) {\n"
  "  ThrI t; t.lo = 0u; t.span = 0xffffffffu; t.invert = false;\n"
  "  const double off = biased ? 2147483648.0 : 0.0;\n"
  "  if (c != c) { t.invert = (op != 4); return t; }\n"
  "  double lo = -1e300, hi = 1e300; bool ne = false;\n"
  "  if (op == 3 || op == 4) { if (floor(c) != c) { t.invert = (op == 3); return t; } lo = c; hi = c; ne = (op == 4); }\n"
  "  else if (op == 5) hi = ceil(c) - 1.0;\n"
  "  else if (op == 7) hi = floor(c);\n"
  "  else if (op == 6) lo = floor(c) + 1.0;\n"
  "  else lo = ceil(c);\n"
  "  lo += off; hi += off;\n"
  "  if (lo < 0.0) lo = 0.0;\n"
  "  if (hi > 4294967295.0) hi = 4294967295.0;\n"
  "  if (lo > hi) { t.invert = !ne; return t; }\n"
  "  t.lo = (u32)lo; t.span = (u32)(hi - lo); t.invert = ne; return t;\n"
  "}\n"
  /* float comparison with bounds rounded down/up from the double literal */
  "struct ThrF { float t; int op; bool strict; __device__ __forceinline__ bool m(float v) const {\n"
  "  if (op == 5) return strict ? v < t : v <= t;\n"
  "  if (op == 7) return v <= t;\n"
  "  if (op == 6) return strict ? v > t : v >= t;\n"
  "  if (op == 8) return v >= t;\n"
  "  if (op == 3) return v == t;\n"
  "  return v != t; } };\n"
  "__device__ ThrF cql_thr_f32(double c, int op) {\n"
  "  ThrF r; r.op = op; r.strict = true; r.t = __int_as_float(0x7fc00000);\n"
  "  if (c != c) return r;\n"
  "  float fd = __double2float_rd(c), fu = __double2float_ru(c);\n"
  "  if (op == 5) { r.t = fd; r.strict = ((double)fd == c); }\n"
  "  else if (op == 7) r.t = fd;\n"
  "  else if (op == 6) { r.t = fu; r.strict = ((double)fu == c); }\n"
  "  else if (op == 8) r.t = fu;\n"
  "  else if ((double)fd == c) r.t = fd;\n"
  "  return r; }\n"
  /* double comparison as an interval of order keys ((bits >> 63) ? ~bits : bits | sign bit): -0.0 and
     +0.0 are neighbouring keys, NaN keys lie beyond the infinities (only != matches a NaN) */
  "struct ThrD { u64 lo, span; bool invert; __device__ __forceinline__ bool m(u64 bits) const {\n"
  "  u64 k = (bits >> 63) ? ~bits : (bits | 0x8000000000000000ull); return ((k - lo) <= span) != invert; } };\n"
  "__device__ __forceinline__ u64 cql_dkey(double x) { u64 b = (u64)__double_as_longlong(x); return (b >> 63) ? ~b : (b | 0x8000000000000000ull); }\n"
  "__device__ ThrD cql_thr_f64(double c, int op) {\n"
  "  ThrD t; t.lo = 0ull; t.span = ~0ull; t.invert = false;\n"
  "  if (c != c) { t.invert = (op != 4); return t; }\n"
  "  const u64 kninf = cql_dkey(__longlong_as_double(0xfff0000000000000ll)), kpinf = cql_dkey(__longlong_as_double(0x7ff0000000000000ll));\n"
  "  const u64 kzn = 0x7fffffffffffffffull, kzp = 0x8000000000000000ull;\n"
  "  const bool zero = c == 0.0; const u64 kc = cql_dkey(c); u64 lo, hi; bool ne = false, empty = false;\n"
  "  if (op == 3 || op == 4) { lo = zero ? kzn : kc; hi = zero ? kzp : kc; ne = (op == 4); }\n"
  "  else if (op == 5) { lo = kninf; hi = zero ? kzn - 1ull : kc - 1ull; empty = (kc == kninf); }\n"
  "  else if (op == 7) { lo = kninf; hi = zero ? kzp : kc; }\n"
  "  else if (op == 6) { lo = zero ? kzp + 1ull : kc + 1ull; hi = kpinf; empty = (kc == kpinf); }\n"
  "  else { lo = zero ? kzn : kc; hi = kpinf; }\n"
  "  if (empty || lo > hi) { t.invert = true; return t; }\n"
  "  t.lo = lo; t.span = hi - lo; t.invert = ne; return t; }\n"
  /* raw strings: the data slot holds bytes, the next slot the row's u64 offsets (scan_filter.comp:105-200) */
  "__device__ __forceinline__ u32 cql_byte(const CqlLaunch& a, u32 slot, u64 i) { const unsigned char* p = (const unsigned char*)a.buf[6 + slot]; return p[i]; }\n"
  "__device__ __forceinline__ u32 cql_cbyte(const CqlLaunch& a, u32 wo, u32 i) { const unsigned char* p = (const unsigned char*)a.buf[2]; return p[wo * 4u + i]; }\n"
  "__device__ __forceinline__ u32 cql_off(const CqlLaunch& a, u32 slot, u64 row) { const u32* o = (const u32*)a.buf[6 + slot + 1]; return o[row * 2]; }\n"
  "__device__ bool cql_str_eq(const CqlLaunch& a, u32 slot, u64 row, u32 wo, u32 len) {\n"
  "  u32 s = cql_off(a, slot, row), e = cql_off(a, slot, row + 1); if (e - s != len) return false;\n"
  "  for (u32 i = 0; i < len; i++) if (cql_byte(a, slot, s + i) != cql_cbyte(a, wo, i)) return false; return true; }\n"
  "__device__ int cql_str_cmp3(const CqlLaunch& a, u32 slot, u64 row, u32 wo, u32 len) {\n"
  "  u32 s = cql_off(a, slot, row), e = cql_off(a, slot, row + 1); u32 n = e - s; u32 m = n < len ? n : len;\n"
  "  for (u32 i = 0; i < m; i++) { u32 x = cql_byte(a, slot, s + i), y = cql_cbyte(a, wo, i); if (x != y) return x < y ? -1 : 1; }\n"
  "  return n < len ? -1 : (n > len ? 1 : 0); }\n"
  "__device__ bool cql_str_contains(const CqlLaunch& a, u32 slot, u64 row, u32 wo, u32 len) {\n"
  "  u32 s = cql_off(a, slot, row), e = cql_off(a, slot, row + 1); u32 n = e - s; if (len == 0) return true; if (n < len) return false;\n"
  "  for (u32 i = 0; i + len <= n; i++) { u32 j = 0; while (j < len && cql_byte(a, slot, s + i + j) == cql_cbyte(a, wo, j)) j++; if (j == len) return true; }\n"
  "  return false; }\n";

/* declarations and loads of the 8 raw rows of every numeric slot the expression reads */
static void emit_loads(Str* out, const int* slot_type)
{
  for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++)
  {
    int t = slot_type[s];
    if (!t) continue;
    int w = type_bytes((uint32_t)t);
    if (w == 8) sprintf_(out, "      u64 r%d[8];\n", s);
    else sprintf_(out, "      u32 r%d[8];\n", s);
  }
  sputs(out, "      if (valid == 8u) {\n");
  for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++)
  {
    int t = slot_type[s];
    if (!t) continue;
    int w = type_bytes((uint32_t)t);
    if (w == 4)
      sprintf_(out,
               "        { const uint4* p = (const uint4*)a.buf[%d] + (row0 >> 2); uint4 q0 = cql_ld4(p), q1 = cql_ld4(p + 1);\n"
               "          r%d[0] = q0.x; r%d[1] = q0.y; r%d[2] = q0.z; r%d[3] = q0.w; r%d[4] = q1.x; r%d[5] = q1.y; r%d[6] = q1.z; r%d[7] = q1.w; }\n",
               6 + s, s, s, s, s, s, s, s, s);
    else if (w == 8)
      sprintf_(out,
               "        { const uint4* p = (const uint4*)a.buf[%d] + (row0 >> 1);\n"
               "          for (int v = 0; v < 4; v++) { uint4 q = cql_ld4(p + v); r%d[2 * v] = ((u64)q.y << 32) | q.x; r%d[2 * v + 1] = ((u64)q.w << 32) | q.z; } }\n",
               6 + s, s, s);
    else
      sprintf_(out,
               "        { uint2 q = *((const uint2*)((const unsigned char*)a.buf[%d] + row0));\n"
               "          for (int v = 0; v < 4; v++) { r%d[v] = (q.x >> (8 * v)) & 0xffu; r%d[v + 4] = (q.y >> (8 * v)) & 0xffu; } }\n",
               6 + s, s, s);
  }
  sputs(out, "      } else {\n");
  for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++)
  {
    int t = slot_type[s];
    if (!t) continue;
    int w = type_bytes((uint32_t)t);
    if (w == 4)
      sprintf_(out, "        for (u32 v = 0; v < 8u; v++) r%d[v] = v < valid ? ((const u32*)a.buf[%d])[row0 + v] : 0u;\n", s, 6 + s);
    else if (w == 8)
      sprintf_(out, "        for (u32 v = 0; v < 8u; v++) r%d[v] = v < valid ? ((const u64*)a.buf[%d])[row0 + v] : 0ull;\n", s, 6 + s);
    else
      sprintf_(out, "        for (u32 v = 0; v < 8u; v++) r%d[v] = v < valid ? (u32)((const unsigned char*)a.buf[%d])[row0 + v] : 0u;\n", s, 6 + s);
  }
  sputs(out, "      }\n");
}

/* accumulate one matching row k into the per-thread aggregates of the fused kernel */
static void emit_fused_accumulate(Str* out, const CqlFusedAgg* f)
{
  for (uint32_t c = 0; c < f->column_count; c++)
  {
    int s = (int)f->slots[c];
    switch (f->coltypes[c])
    {
      case CQLOPS_TYPE_U32:
        sprintf_(out, "          { u32 x = r%d[k]; us%u += x; un%u = min(un%u, x); ux%u = max(ux%u, x); }\n", s, c, c, c, c, c);
        break;
      case CQLOPS_TYPE_I32:
        sprintf_(out, "          { int x = (int)r%d[k]; is%u += x; in%u = min(in%u, x); ix%u = max(ix%u, x); }\n", s, c, c, c, c, c);
        break;
      case CQLOPS_TYPE_F32:
        sprintf_(out, "          { float x = __uint_as_float(r%d[k]); ds%u += (double)x; fn%u = fminf(fn%u, x); fx%u = fmaxf(fx%u, x); }\n", s, c, c, c,
                 c, c);
        break;
      default:
      {
        char* d = dbl_of(s, (int)f->coltypes[c]);
        sprintf_(out, "          { double x = %s; ds%u += x; dn%u = fmin(dn%u, x); dx%u = fmax(dx%u, x); }\n", d, c, c, c, c, c);
        free(d);
      }
    }
  }
}

int cqlops_program_source(const CqlProgram* prog, uint32_t kind, const CqlFusedAgg* fuse, char* out, uint64_t cap, uint64_t* out_len)
{
  Gen g;
  memset(&g, 0, sizeof(g));
  g.prog = prog;
  for (uint64_t ip = 0; ip < prog->word_count; ip++)
  {
    uint32_t op = prog->words[ip];
    if (op >= OP_STR_EQ && op != OP_HALT && op != OP_PUSH_FALSE) g.uses_strings = 1;
  }
  /* the fused kernels read their aggregate columns too */
  if (fuse && kind != CQLOPS_KERNEL_SCAN)
  {
    for (uint32_t c = 0; c < fuse->column_count; c++) note_slot(&g, (int)fuse->slots[c], (int)fuse->coltypes[c]);
    if (kind == CQLOPS_KERNEL_FUSED_GROUP)
      for (uint32_t k = 0; k < fuse->key_count; k++) note_slot(&g, (int)fuse->key_slots[k], (int)fuse->key_types[k]);
  }
  char* expr = build_expression(&g);
  if (g.failed || !expr)
  {
    free(expr);
    free(g.pro.p);
    if (out && cap) snprintf(out, cap, "%s", g.why);
    return 0;
  }
  Str s;
  memset(&s, 0, sizeof(s));
  if (kind == CQLOPS_KERNEL_FUSED_GROUP)
  {
    uint32_t width = 2 + 4 * fuse->column_count;
    uint32_t table = fuse->group_count * width;
    uint32_t copies = 1;
    while (copies < 8 && (uint64_t)table * 4 * copies * 2 <= 48 * 1024) copies *= 2;
    sprintf_(&s, "// cql: block=256 smem=%u per_sm=6\n", table * 4 * copies);
  }
  else sputs(&s, "// cql: block=256 smem=0 per_sm=6\n");
  sputs(&s, PRELUDE);
  sputs(&s, "extern \"C\" __global__ void __launch_bounds__(256) cql_main(CqlLaunch a)\n{\n");
  sputs(&s, "  const u64 rows = cql_word(a, 0);\n");
  sputs(&s, g.pro.p ? g.pro.p : "");
  sputs(&s, "  const u64 groups8 = (rows + 7ull) / 8ull;\n  const u64 per_pass = (u64)gridDim.x * 256ull;\n");
  sputs(&s, "  const u32 lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;\n");

  if (kind == CQLOPS_KERNEL_SCAN)
  {
    sputs(&s,
          "  __shared__ u32 s_warp[8]; __shared__ u32 s_base;\n"
          "  u32* out = (u32*)a.buf[3]; u32* out_count = (u32*)a.buf[4]; const u32* skip = (const u32*)a.buf[5];\n"
          "  const u64 capacity = a.bytes[3] / 8ull; const u32 skip_shift = cql_word(a, 6); const bool skip_on = cql_word(a, 8) != 0u;\n"
          "  const bool bitmap_mode = cql_word(a, 10) != 0u; const u64 bitmap_words = a.bytes[3] / 4ull; u32 bitmap_count = 0u;\n"
          "  for (u64 base = (u64)blockIdx.x * 256ull; base < groups8; base += per_pass)\n  {\n"
          "    const u64 row0 = (base + threadIdx.x) * 8ull;\n"
          "    const u32 valid = row0 < rows ? (u32)min((u64)8, rows - row0) : 0u;\n"
          "    u32 live = 0u;\n"
          "    bool go = valid != 0u;\n"
          "    if (go && skip_on) { u64 ch = row0 >> skip_shift; go = ((skip[ch >> 5] >> (ch & 31ull)) & 1u) == 0u; }\n"
          "    if (go)\n    {\n");
    emit_loads(&s, g.slot_type);
    sprintf_(&s, "#pragma unroll\n      for (u32 k = 0; k < 8u; k++) { if (k < valid) { bool m = %s; live |= (m ? 1u : 0u) << k; } }\n", expr);
    sputs(&s,
          "    }\n"
          "    if (bitmap_mode)\n    {\n"
          "      u32 m = live << (8u * (lane & 3u)); m |= __shfl_xor_sync(0xffffffffu, m, 1); m |= __shfl_xor_sync(0xffffffffu, m, 2);\n"
          "      const u64 word = (base + threadIdx.x) >> 2;\n"
          "      if ((lane & 3u) == 0u && word < bitmap_words) out[word] = m;\n"
          "      bitmap_count += __popc(live);\n"
          "      continue;\n    }\n"
          "    const u32 n = __popc(live); u32 incl = n;\n"
          "#pragma unroll\n    for (int o = 1; o < 32; o <<= 1) { u32 y = __shfl_up_sync(0xffffffffu, incl, o); if (lane >= (u32)o) incl += y; }\n"
          "    if (lane == 31u) s_warp[warp] = incl;\n"
          "    __syncthreads();\n"
          "    if (threadIdx.x == 0u) { u32 run = 0u; for (int w = 0; w < 8; w++) { u32 t = s_warp[w]; s_warp[w] = run; run += t; } s_base = run ? atomicAdd(out_count, run) : 0u; }\n"
          "    __syncthreads();\n"
          "    u64 pos = (u64)s_base + s_warp[warp] + (incl - n);\n"
          "    while (live) { u32 k = __ffs(live) - 1u; live &= live - 1u; if (pos < capacity) { uint2 pr = make_uint2((u32)(row0 + k), 0u); *((uint2*)(out + pos * 2ull)) = pr; } pos++; }\n"
          "    __syncthreads();\n"
          "  }\n"
          "  if (bitmap_mode)\n  {\n"
          "#pragma unroll\n    for (int o = 16; o > 0; o >>= 1) bitmap_count += __shfl_xor_sync(0xffffffffu, bitmap_count, o);\n"
          "    if (lane == 0u && bitmap_count) atomicAdd(out_count, bitmap_count);\n  }\n}\n");
  }
  else if (kind == CQLOPS_KERNEL_FUSED_AGG)
  {
    uint32_t kc = fuse->column_count;
    sputs(&s, "  u32 cnt = 0u;\n");
    for (uint32_t c = 0; c < kc; c++)
    {
      switch (fuse->coltypes[c])
      {
        case CQLOPS_TYPE_U32: sprintf_(&s, "  u64 us%u = 0ull; u32 un%u = 0xffffffffu, ux%u = 0u;\n", c, c, c); break;
        case CQLOPS_TYPE_I32: sprintf_(&s, "  long long is%u = 0ll; int in%u = 0x7fffffff, ix%u = (int)0x80000000;\n", c, c, c); break;
        case CQLOPS_TYPE_F32: sprintf_(&s, "  double ds%u = 0.0; float fn%u = __int_as_float(0x7f7fffff), fx%u = -__int_as_float(0x7f7fffff);\n", c, c, c); break;
        default: sprintf_(&s, "  double ds%u = 0.0, dn%u = 1.7976931348623157e308, dx%u = -1.7976931348623157e308;\n", c, c, c);
      }
    }
    sputs(&s,
          "  for (u64 base = (u64)blockIdx.x * 256ull; base < groups8; base += per_pass)\n  {\n"
          "    const u64 row0 = (base + threadIdx.x) * 8ull;\n"
          "    const u32 valid = row0 < rows ? (u32)min((u64)8, rows - row0) : 0u;\n"
          "    if (valid != 0u)\n    {\n");
    emit_loads(&s, g.slot_type);
    sprintf_(&s, "#pragma unroll\n      for (u32 k = 0; k < 8u; k++)\n      {\n        if (k < valid && (%s))\n        {\n          cnt += 1u;\n", expr);
    emit_fused_accumulate(&s, fuse);
    sputs(&s, "        }\n      }\n    }\n  }\n");
    /* block reduction and the partials */
    sputs(&s,
          "  __shared__ double sh_d[8]; __shared__ unsigned long long sh_u[8]; __shared__ u32 sh_w[8]; __shared__ float sh_f[8];\n"
          "  double* partials = (double*)a.buf[3]; const u64 pcap = a.bytes[3] / 8ull; const u32 wgs = cql_word(a, 12);\n");
    sprintf_(&s, "  const u32 width = %uu;\n", 1 + 3 * kc);
    sputs(&s,
          "  unsigned long long tc = cnt;\n"
          "  for (int o = 16; o > 0; o >>= 1) tc += __shfl_xor_sync(0xffffffffu, tc, o);\n"
          "  if (lane == 0u) sh_u[warp] = tc; __syncthreads();\n"
          "  if (threadIdx.x == 0u) { unsigned long long t = 0; for (int w = 0; w < 8; w++) t += sh_u[w]; sh_u[0] = t; } __syncthreads();\n"
          "  const unsigned long long block_count = sh_u[0]; __syncthreads();\n"
          "  const u64 at = (u64)blockIdx.x * width;\n"
          "  if (threadIdx.x == 0u && at < pcap) partials[at] = (double)block_count;\n");
    for (uint32_t c = 0; c < kc; c++)
    {
      uint32_t t = fuse->coltypes[c];
      const char* fold;
      if (t == CQLOPS_TYPE_U32)
        fold = "  { unsigned long long s_ = us%u; u32 n_ = un%u, x_ = ux%u;\n"
               "    for (int o = 16; o > 0; o >>= 1) { s_ += __shfl_xor_sync(0xffffffffu, s_, o); n_ = min(n_, __shfl_xor_sync(0xffffffffu, n_, o)); x_ = max(x_, __shfl_xor_sync(0xffffffffu, x_, o)); }\n"
               "    if (lane == 0u) { sh_u[warp] = s_; sh_w[warp] = n_; } __syncthreads();\n"
               "    if (threadIdx.x == 0u) { for (int w = 1; w < 8; w++) { s_ += sh_u[w]; n_ = min(n_, sh_w[w]); } sh_u[0] = s_; sh_w[0] = n_; } __syncthreads();\n"
               "    double S = (double)sh_u[0], N = (double)sh_w[0]; __syncthreads();\n"
               "    if (lane == 0u) sh_w[warp] = x_; __syncthreads();\n"
               "    if (threadIdx.x == 0u) { for (int w = 1; w < 8; w++) x_ = max(x_, sh_w[w]); sh_w[0] = x_; } __syncthreads();\n"
               "    double X = (double)sh_w[0]; __syncthreads();\n"
               "    if (threadIdx.x == 0u && at + %u + 2 < pcap) { partials[at + %u] = S; partials[at + %u + 1] = block_count ? N : 1.7976931348623157e308; partials[at + %u + 2] = block_count ? X : -1.7976931348623157e308; } }\n";
      else if (t == CQLOPS_TYPE_I32)
        fold = "  { long long s_ = is%u; int n_ = in%u, x_ = ix%u;\n"
               "    for (int o = 16; o > 0; o >>= 1) { s_ += __shfl_xor_sync(0xffffffffu, s_, o); n_ = min(n_, __shfl_xor_sync(0xffffffffu, n_, o)); x_ = max(x_, __shfl_xor_sync(0xffffffffu, x_, o)); }\n"
               "    if (lane == 0u) { sh_u[warp] = (unsigned long long)s_; sh_w[warp] = (u32)n_; } __syncthreads();\n"
               "    if (threadIdx.x == 0u) { for (int w = 1; w < 8; w++) { s_ += (long long)sh_u[w]; n_ = min(n_, (int)sh_w[w]); } sh_u[0] = (unsigned long long)s_; sh_w[0] = (u32)n_; } __syncthreads();\n"
               "    double S = (double)(long long)sh_u[0], N = (double)(int)sh_w[0]; __syncthreads();\n"
               "    if (lane == 0u) sh_w[warp] = (u32)x_; __syncthreads();\n"
               "    if (threadIdx.x == 0u) { for (int w = 1; w < 8; w++) x_ = max(x_, (int)sh_w[w]); sh_w[0] = (u32)x_; } __syncthreads();\n"
               "    double X = (double)(int)sh_w[0]; __syncthreads();\n"
               "    if (threadIdx.x == 0u && at + %u + 2 < pcap) { partials[at + %u] = S; partials[at + %u + 1] = block_count ? N : 1.7976931348623157e308; partials[at + %u + 2] = block_count ? X : -1.7976931348623157e308; } }\n";
      else if (t == CQLOPS_TYPE_F32)
        fold = "  { double s_ = ds%u; float n_ = fn%u, x_ = fx%u;\n"
               "    for (int o = 16; o > 0; o >>= 1) { s_ += __shfl_xor_sync(0xffffffffu, s_, o); n_ = fminf(n_, __shfl_xor_sync(0xffffffffu, n_, o)); x_ = fmaxf(x_, __shfl_xor_sync(0xffffffffu, x_, o)); }\n"
               "    if (lane == 0u) { sh_d[warp] = s_; sh_f[warp] = n_; } __syncthreads();\n"
               "    if (threadIdx.x == 0u) { for (int w = 1; w < 8; w++) { s_ += sh_d[w]; n_ = fminf(n_, sh_f[w]); } sh_d[0] = s_; sh_f[0] = n_; } __syncthreads();\n"
               "    double S = sh_d[0], N = (double)sh_f[0]; __syncthreads();\n"
               "    if (lane == 0u) sh_f[warp] = x_; __syncthreads();\n"
               "    if (threadIdx.x == 0u) { for (int w = 1; w < 8; w++) x_ = fmaxf(x_, sh_f[w]); sh_f[0] = x_; } __syncthreads();\n"
               "    double X = (double)sh_f[0]; __syncthreads();\n"
               "    if (threadIdx.x == 0u && at + %u + 2 < pcap) { partials[at + %u] = S; partials[at + %u + 1] = block_count ? N : 1.7976931348623157e308; partials[at + %u + 2] = block_count ? X : -1.7976931348623157e308; } }\n";
      else
        fold = "  { double s_ = ds%u, n_ = dn%u, x_ = dx%u;\n"
               "    for (int o = 16; o > 0; o >>= 1) { s_ += __shfl_xor_sync(0xffffffffu, s_, o); n_ = fmin(n_, __shfl_xor_sync(0xffffffffu, n_, o)); x_ = fmax(x_, __shfl_xor_sync(0xffffffffu, x_, o)); }\n"
               "    if (lane == 0u) sh_d[warp] = s_; __syncthreads();\n"
               "    if (threadIdx.x == 0u) { for (int w = 1; w < 8; w++) s_ += sh_d[w]; sh_d[0] = s_; } __syncthreads();\n"
               "    double S = sh_d[0]; __syncthreads();\n"
               "    if (lane == 0u) sh_d[warp] = n_; __syncthreads();\n"
               "    if (threadIdx.x == 0u) { for (int w = 1; w < 8; w++) n_ = fmin(n_, sh_d[w]); sh_d[0] = n_; } __syncthreads();\n"
               "    double N = sh_d[0]; __syncthreads();\n"
               "    if (lane == 0u) sh_d[warp] = x_; __syncthreads();\n"
               "    if (threadIdx.x == 0u) { for (int w = 1; w < 8; w++) x_ = fmax(x_, sh_d[w]); sh_d[0] = x_; } __syncthreads();\n"
               "    double X = sh_d[0]; __syncthreads();\n"
               "    if (threadIdx.x == 0u && at + %u + 2 < pcap) { partials[at + %u] = S; partials[at + %u + 1] = N; partials[at + %u + 2] = X; } }\n";
      sprintf_(&s, fold, c, c, c, 1 + 3 * c, 1 + 3 * c, 1 + 3 * c, 1 + 3 * c);
    }
    /* workgroups of the reference's grid this launch did not cover: neutral partials */
    sputs(&s,
          "  for (u64 w = gridDim.x + blockIdx.x; w < wgs; w += gridDim.x)\n"
          "    for (u32 i = threadIdx.x; i < width; i += 256u)\n"
          "    {\n"
          "      u64 at2 = w * width + i; if (at2 >= pcap) continue;\n"
          "      u32 part = i == 0u ? 0u : (i - 1u) % 3u;\n"
          "      partials[at2] = (i == 0u || part == 0u) ? 0.0 : (part == 1u ? 1.7976931348623157e308 : -1.7976931348623157e308);\n"
          "    }\n}\n");
  }
  else
  {
    /* grouped: up to 3 keys as digits, 2 + 4k words per group, per-warp copies of the table in shared memory */
    uint32_t kc = fuse->column_count;
    uint32_t width = 2 + 4 * kc;
    uint32_t table = fuse->group_count * width;
    uint32_t copies = 1;
    while (copies < 8 && (uint64_t)table * 4 * copies * 2 <= 48 * 1024) copies *= 2;
    sprintf_(&s, "  extern __shared__ u32 s_acc[];\n  const u32 WIDTH = %uu, GROUPS = %uu, COPIES = %uu;\n", width, fuse->group_count, copies);
    sputs(&s,
          "  for (u32 i = threadIdx.x; i < GROUPS * WIDTH * COPIES; i += 256u) { u32 f = (i % (GROUPS * WIDTH)) % WIDTH; bool is_min = f == 1u || (f >= 2u && ((f - 2u) % 4u) == 2u); s_acc[i] = is_min ? 0xffffffffu : 0u; }\n"
          "  __syncthreads();\n"
          "  u32* acc = s_acc + (warp % COPIES) * GROUPS * WIDTH;\n");
    const uint32_t min_words[3] = { 14, 15, 13 };
    for (uint32_t k = 0; k < fuse->key_count; k++) sprintf_(&s, "  const int KM%u = (int)cql_word(a, %uu);\n", k, min_words[k]);
    sputs(&s,
          "  for (u64 base = (u64)blockIdx.x * 256ull; base < groups8; base += per_pass)\n  {\n"
          "    const u64 row0 = (base + threadIdx.x) * 8ull;\n"
          "    const u32 valid = row0 < rows ? (u32)min((u64)8, rows - row0) : 0u;\n"
          "    if (valid != 0u)\n    {\n");
    emit_loads(&s, g.slot_type);
    sprintf_(&s, "#pragma unroll\n      for (u32 k = 0; k < 8u; k++)\n      {\n        if (k < valid && (%s))\n        {\n          u32 g = 0u; bool key_ok = true;\n", expr);
    for (uint32_t k = 0; k < fuse->key_count; k++)
    {
      char* d = dbl_of((int)fuse->key_slots[k], (int)fuse->key_types[k]);
      sprintf_(&s, "          { int part = (int)(%s) - KM%u; key_ok = key_ok && part >= 0 && (u32)part < %uu; g = g * %uu + (u32)part; }\n", d, k,
               fuse->key_ranges[k], fuse->key_ranges[k]);
      free(d);
    }
    sputs(&s,
          "          if (key_ok && g < GROUPS)\n          {\n"
          "            u32* b = acc + g * WIDTH;\n"
          "            atomicAdd(&b[0], 1u); atomicMin(&b[1], (u32)(row0 + k));\n");
    for (uint32_t c = 0; c < kc; c++)
    {
      int sg = fuse->coltypes[c] == CQLOPS_TYPE_I32;
      sprintf_(&s,
               "            { u32 u = r%u[k]%s; u32 old = atomicAdd(&b[%u], u); if (old + u < old) atomicAdd(&b[%u], 1u); atomicMin(&b[%u], u); atomicMax(&b[%u], u); }\n",
               fuse->slots[c], sg ? " ^ 0x80000000u" : "", 2 + 4 * c, 3 + 4 * c, 4 + 4 * c, 5 + 4 * c);
    }
    sputs(&s, "          }\n        }\n      }\n    }\n  }\n  __syncthreads();\n");
    sputs(&s,
          "  u32* out_words = (u32*)a.buf[3]; const u64 ocap = a.bytes[3] / 4ull;\n"
          "  for (u32 g = threadIdx.x; g < GROUPS; g += 256u)\n  {\n"
          "    u32 count = 0u, minrow = 0xffffffffu;\n"
          "    for (u32 c = 0; c < COPIES; c++) { const u32* b = s_acc + (c * GROUPS + g) * WIDTH; count += b[0]; minrow = min(minrow, b[1]); }\n"
          "    if (count == 0u || (u64)(g + 1) * WIDTH > ocap) continue;\n"
          "    u32* o = out_words + (u64)g * WIDTH;\n"
          "    atomicAdd(&o[0], count); atomicMin(&o[1], minrow);\n");
    for (uint32_t c = 0; c < kc; c++)
    {
      sprintf_(&s,
               "    { u64 sum = 0ull; u32 mn = 0xffffffffu, mx = 0u;\n"
               "      for (u32 c = 0; c < COPIES; c++) { const u32* b = s_acc + (c * GROUPS + g) * WIDTH; sum += ((u64)b[%u] << 32) | b[%u]; mn = min(mn, b[%u]); mx = max(mx, b[%u]); }\n"
               "      atomicAdd((unsigned long long*)&o[%u], (unsigned long long)sum); atomicMin(&o[%u], mn); atomicMax(&o[%u], mx); }\n",
               3 + 4 * c, 2 + 4 * c, 4 + 4 * c, 5 + 4 * c, 2 + 4 * c, 4 + 4 * c, 5 + 4 * c);
    }
    sputs(&s, "  }\n}\n");
  }
  free(expr);
  free(g.pro.p);
  if (s.failed)
  {
    free(s.p);
    return 0;
  }
  if (out_len) *out_len = s.n;
  int ok = 1;
  if (out)
  {
    if (s.n + 1 > cap) ok = 0;
    else memcpy(out, s.p, s.n + 1);
  }
  free(s.p);
  return ok;
}

int cql_codegen_batch_predicate(const CqlProgram* prog, CqlBatchSite* sites, uint32_t site_cap, uint32_t* site_count, int* slot_type,
                                char** expr, char* why, size_t why_cap)
{
  Gen g;
  memset(&g, 0, sizeof(g));
  g.prog = prog;
  g.batch = 1;
  g.batch_sites = sites;
  g.batch_cap = site_cap;
  char* e = build_expression(&g);
  free(g.pro.p);
  if (g.failed || !e)
  {
    free(e);
    if (why && why_cap) snprintf(why, why_cap, "%s", g.failed ? g.why : "empty program");
    return 0;
  }
  *site_count = (uint32_t)g.sites;
  for (int i = 0; i < CQLOPS_MAX_BINDINGS; i++) slot_type[i] = g.slot_type[i];
  *expr = e;
  return 1;
}
