/*
 * cql_batch.c - many filter/aggregate queries over one table in one shared scan.
 *
 * SELECT COUNT(*), SUM(col) FROM t WHERE <query q's condition>, for q = 0 .. Q-1, answered by one pass
 * over the table: the batched form of the per-query fused filter+aggregate (qe_fused_filter_aggregate,
 * src/query_exec/query_exec.c:9888-10254, generated kernel query_kernel.c:1538-1614).
 *
 *  1. Each query's program is rebound so that every column is read from the register block of its
 *     column index, and queries whose rebound bytecode is the same word for word share a shape. The
 *     shape is emitted once as a predicate (cql_codegen_batch_predicate) and evaluated for each of its
 *     queries; a shape's literals differ per query only.
 *  2. The literals of a comparison with a column become per-query thresholds on the host: an interval
 *     of (sign-biased) codes for whole-number columns and of order keys for f64 columns, float bounds
 *     rounded down/up for f32 columns - integer work per row, the same answer as the reference's
 *     comparison in double.
 *  3. SUM is accumulated exactly in integers of the value scaled by 2^k, k chosen from the column's range
 *     and the rows one warp can see so that a warp's total stays below 2^62: the sum of the matched rows
 *     is then exact up to 2^-(k+1) per row, independent of order (for the configured tables, far below
 *     1e-16 of the largest value).
 *  4. One warp owns its accumulators in shared memory (a 32-bit count and a 64-bit sum per query, no
 *     atomics); a CTA folds its warps into 128-bit sums, a second kernel folds the CTAs in order. At
 *     most CQL_BATCH_LAUNCH_QUERIES queries go into one launch.
 */
#define _POSIX_C_SOURCE 200809L
#include "cqlops.h"
#include "cql_ops_internal.h"
#include "cql_codegen.h"

#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define QE_GPU_WORKGROUP_SIZE 256
#define BATCH_MAX_SITES 16
#define BATCH_MAX_CONSTS 32
#define CQL_BATCH_LAUNCH_QUERIES 384
#define BATCH_CTAS_PER_SM 6
#define BATCH_MAX_SHAPES 256
#define CQL_BATCH_CATALOG_SHAPES 64

static int refuse(const char* why)
{
  cqlops_note_error(why);
  return 0;
}

enum
{
  OP_LOAD_NUM_COL = 1, OP_PUSH_CONST = 2, OP_CMP_EQ = 3, OP_CMP_NE = 4, OP_CMP_LT = 5, OP_CMP_GT = 6, OP_CMP_LE = 7, OP_CMP_GE = 8,
  OP_STR_EQ = 11, OP_STR_CONTAINS = 12, OP_TRIGRAM_SIM = 15, OP_EDIT_DISTANCE = 16, OP_STR_NE = 17, OP_STR_GE = 21,
};

/* a threshold, 32 bytes: a/b the interval (low, span), c = invert (or the op of a float test), d = strict */
typedef struct
{
  uint64_t a, b;
  uint32_t c, d;
  uint64_t pad;
} Thr;

/* ---- thresholds, worked out on the host ---- */

/* whole-number column: match = ((code - lo) <= span) != invert over the (sign-biased) 32-bit code; the
   same rules as the per-query kernel's cql_thr_int */
static void thr_int(double c, int op, int biased, Thr* t)
{
  memset(t, 0, sizeof(*t));
  t->b = 0xffffffffu;
  double off = biased ? 2147483648.0 : 0.0;
  if (c != c)
  {
    t->c = op != OP_CMP_NE;
    return;
  }
  double lo = -1e300, hi = 1e300;
  int ne = 0;
  if (op == OP_CMP_EQ || op == OP_CMP_NE)
  {
    if (floor(c) != c)
    {
      t->c = op == OP_CMP_EQ;
      return;
    }
    lo = c;
    hi = c;
    ne = op == OP_CMP_NE;
  }
  else if (op == OP_CMP_LT) hi = ceil(c) - 1.0;
  else if (op == OP_CMP_LE) hi = floor(c);
  else if (op == OP_CMP_GT) lo = floor(c) + 1.0;
  else lo = ceil(c);
  lo += off;
  hi += off;
  if (lo < 0.0) lo = 0.0;
  if (hi > 4294967295.0) hi = 4294967295.0;
  if (lo > hi)
  {
    t->c = !ne;
    return;
  }
  t->a = (uint32_t)lo;
  t->b = (uint32_t)(hi - lo);
  t->c = (uint32_t)ne;
}

static float f32_down(double c)
{
  float f = (float)c;
  if ((double)f > c) f = nextafterf(f, -INFINITY);
  return f;
}

static float f32_up(double c)
{
  float f = (float)c;
  if ((double)f < c) f = nextafterf(f, INFINITY);
  return f;
}

/* f32 column: the literal rounded down/up to floats, as the per-query kernel's cql_thr_f32 */
static void thr_f32(double c, int op, Thr* t)
{
  memset(t, 0, sizeof(*t));
  float v = NAN;
  uint32_t strict = 1;
  if (c == c)
  {
    float fd = f32_down(c), fu = f32_up(c);
    if (op == OP_CMP_LT)
    {
      v = fd;
      strict = (double)fd == c;
    }
    else if (op == OP_CMP_LE) v = fd;
    else if (op == OP_CMP_GT)
    {
      v = fu;
      strict = (double)fu == c;
    }
    else if (op == OP_CMP_GE) v = fu;
    else if ((double)fd == c) v = fd;
  }
  uint32_t bits;
  memcpy(&bits, &v, 4);
  t->a = bits;
  t->c = (uint32_t)op;
  t->d = strict;
}

static uint64_t f64_key(double x)
{
  uint64_t b;
  memcpy(&b, &x, 8);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

/* f64 column: an interval of order keys ((bits >> 63) ? ~bits : bits | sign bit). -0.0 and +0.0 have
   neighbouring keys, which the intervals of a zero literal cover together; NaN keys lie beyond the
   infinities, outside every interval (so only != matches a NaN, as in double). */
static void thr_f64(double c, int op, Thr* t)
{
  memset(t, 0, sizeof(*t));
  const uint64_t kninf = f64_key(-INFINITY), kpinf = f64_key(INFINITY);
  const uint64_t kz_neg = 0x7fffffffffffffffull, kz_pos = 0x8000000000000000ull;
  if (c != c)
  {
    t->b = ~0ull;
    t->c = op != OP_CMP_NE;
    return;
  }
  int zero = c == 0.0;
  uint64_t kc = f64_key(c);
  uint64_t lo, hi;
  int ne = 0;
  switch (op)
  {
    case OP_CMP_EQ: case OP_CMP_NE:
      lo = zero ? kz_neg : kc;
      hi = zero ? kz_pos : kc;
      ne = op == OP_CMP_NE;
      break;
    case OP_CMP_LT:
      lo = kninf;
      hi = zero ? kz_neg - 1 : kc - 1;
      if (c == -INFINITY) lo = 1, hi = 0;
      break;
    case OP_CMP_LE:
      lo = kninf;
      hi = zero ? kz_pos : kc;
      break;
    case OP_CMP_GT:
      lo = zero ? kz_pos + 1 : kc + 1;
      hi = kpinf;
      if (c == INFINITY) lo = 1, hi = 0;
      break;
    default:
      lo = zero ? kz_neg : kc;
      hi = kpinf;
      break;
  }
  if (lo > hi)
  {
    /* nothing matches: the inverted full range */
    t->a = 0;
    t->b = ~0ull;
    t->c = 1;
    return;
  }
  t->a = lo;
  t->b = hi - lo;
  t->c = (uint32_t)ne;
}

static double const_value(const CqlProgram* p, uint32_t index)
{
  uint64_t bits = ((uint64_t)p->consts[2 * index + 1] << 32) | p->consts[2 * index];
  double v;
  memcpy(&v, &bits, 8);
  return v;
}

/* the program with each column load reading the register block of its column index */
static int rebind(const CqlProgram* p, uint32_t column_count, CqlProgram* out)
{
  /* only what the batched predicate reads: the words and the constants (a program is ~80 KB with its
     string pool, which a batched program never uses) */
  if (p->word_count > CQLOPS_MAX_WORDS || p->const_count > CQLOPS_MAX_CONSTS) return 0;
  memcpy(out->words, p->words, p->word_count * sizeof(uint32_t));
  memcpy(out->consts, p->consts, p->const_count * 2 * sizeof(uint32_t));
  out->word_count = p->word_count;
  out->const_count = p->const_count;
  out->str_pool_size = 0;
  out->binding_count = p->binding_count;
  memcpy(out->binding_column, p->binding_column, sizeof(p->binding_column));
  memcpy(out->binding_type, p->binding_type, sizeof(p->binding_type));
  memcpy(out->binding_slot, p->binding_slot, sizeof(p->binding_slot));
  memcpy(out->binding_dict, p->binding_dict, sizeof(p->binding_dict));
  out->next_slot = p->next_slot;
  out->requires_cpu_scan = p->requires_cpu_scan;
  out->has_score_output = p->has_score_output;
  out->error[0] = 0;
  int slot_column[CQLOPS_MAX_BINDINGS];
  for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++) slot_column[s] = -1;
  for (uint32_t b = 0; b < p->binding_count; b++)
    if (p->binding_slot[b] < CQLOPS_MAX_BINDINGS) slot_column[p->binding_slot[b]] = (int)p->binding_column[b];
  uint64_t ip = 0;
  while (ip < p->word_count)
  {
    uint32_t op = p->words[ip++];
    if (op == OP_LOAD_NUM_COL)
    {
      if (ip >= p->word_count) return 0;
      uint32_t operand = p->words[ip];
      uint32_t slot = operand & 0xffu;
      if (slot >= CQLOPS_MAX_BINDINGS || slot_column[slot] < 0 || (uint32_t)slot_column[slot] >= column_count) return 0;
      out->words[ip] = (operand & ~0xffu) | (uint32_t)slot_column[slot];
      ip++;
    }
    else if (op == OP_PUSH_CONST) ip++;
    else if ((op >= OP_STR_EQ && op <= OP_STR_CONTAINS) || (op >= OP_STR_NE && op <= OP_STR_GE) || op == OP_TRIGRAM_SIM || op == OP_EDIT_DISTANCE)
      return 0;
  }
  return 1;
}

static uint64_t words_hash(const CqlProgram* p)
{
  uint64_t h = 1469598103934665603ull;
  for (uint32_t i = 0; i < p->word_count; i++) h = (h ^ p->words[i]) * 1099511628211ull;
  return h ^ p->word_count;
}

/* ---- the generated kernel ---- */

typedef struct
{
  char* p;
  size_t n, cap;
  int failed;
} Buf;

static void bput(Buf* b, const char* fmt, ...)
{
  if (b->failed) return;
  va_list ap;
  for (;;)
  {
    va_start(ap, fmt);
    int need = vsnprintf(b->p ? b->p + b->n : NULL, b->p ? b->cap - b->n : 0, fmt, ap);
    va_end(ap);
    if (need < 0)
    {
      b->failed = 1;
      return;
    }
    if (b->p && b->n + (size_t)need < b->cap)
    {
      b->n += (size_t)need;
      return;
    }
    size_t nc = (b->cap ? b->cap * 2 : 16384) + (size_t)need;
    char* q = (char*)realloc(b->p, nc);
    if (!q)
    {
      b->failed = 1;
      return;
    }
    b->p = q;
    b->cap = nc;
  }
}

static int type_bytes(int t)
{
  if (t == CQLOPS_TYPE_F64 || t == CQLOPS_TYPE_U64 || t == CQLOPS_TYPE_I64) return 8;
  if (t == CQLOPS_TYPE_BOOL) return 1;
  return 4;
}

static const char* BATCH_PRELUDE =
  "typedef unsigned int u32;\n"
  "typedef unsigned long long u64;\n"
  "struct CqlLaunch { void* buf[16]; u64 bytes[16]; u64 push[8]; };\n"
  "struct Thr { u64 a, b; u32 c, d; u64 pad; };\n"
  "__device__ __forceinline__ u32 cql_word(const CqlLaunch& a, u32 i) { u64 s = a.push[i >> 1]; return (i & 1u) ? (u32)(s >> 32) : (u32)s; }\n"
  "__device__ __forceinline__ uint4 cql_ld4(const void* p) { uint4 v; asm volatile(\"ld.global.cs.v4.u32 {%0,%1,%2,%3}, [%4];\" : \"=r\"(v.x), \"=r\"(v.y), \"=r\"(v.z), \"=r\"(v.w) : \"l\"(p)); return v; }\n"
  "__device__ __forceinline__ bool cql_bi(const Thr* t, u32 code) { return ((code - (u32)t->a) <= (u32)t->b) != (t->c != 0u); }\n"
  "__device__ __forceinline__ u64 cql_key(u64 bits) { return (bits >> 63) ? ~bits : (bits | 0x8000000000000000ull); }\n"
  "__device__ __forceinline__ bool cql_bk(const Thr* t, u64 key) { return ((key - t->a) <= t->b) != (t->c != 0u); }\n"
  "__device__ __forceinline__ bool cql_bf(const Thr* t, float v) { float x = __uint_as_float((u32)t->a); u32 op = t->c; bool s = t->d != 0u;\n"
  "  if (op == 5u) return s ? v < x : v <= x; if (op == 7u) return v <= x; if (op == 6u) return s ? v > x : v >= x; if (op == 8u) return v >= x;\n"
  "  if (op == 3u) return v == x; return v != x; }\n"
  /* the warp's sum of a 64-bit value, mod 2^64: four independent warp reductions of its 16-bit slices (a
     32-lane sum of 16-bit values fits in 21 bits), instead of a chain of five 64-bit shuffles and adds */
  "__device__ __forceinline__ long long cql_wsum64(long long v) { const u64 u = (u64)v;\n"
  "  const u64 s0 = __reduce_add_sync(0xffffffffu, (u32)(u & 0xffffu)), s1 = __reduce_add_sync(0xffffffffu, (u32)((u >> 16) & 0xffffu));\n"
  "  const u64 s2 = __reduce_add_sync(0xffffffffu, (u32)((u >> 32) & 0xffffu)), s3 = __reduce_add_sync(0xffffffffu, (u32)(u >> 48));\n"
  "  return (long long)(s0 + (s1 << 16) + (s2 << 32) + (s3 << 48)); }\n"
  "__device__ __forceinline__ double cql_i64d(u64 x) { double u = (double)(u32)(x >> 32) * 4294967296.0 + (double)(u32)x; return (x >> 63) ? u - 18446744073709551616.0 : u; }\n"
  /* x * 2^sh rounded to the nearest integer (ties to even), from the bits of x in integer arithmetic:
     x = m * 2^e, so x * 2^sh = m * 2^(e + sh). Exact, as the product of x by the power of two is; a
     NaN, an infinity or a product past 2^62 takes the double multiply and conversion instead. */
  "__device__ __forceinline__ long long cql_fx64(u64 bits, int sh, double sc)\n"
  "{\n"
  "  const u32 ex = (u32)(bits >> 52) & 0x7ffu;\n"
  "  u64 m = bits & 0xfffffffffffffull;\n"
  "  int e = -1074;\n"
  "  if (ex) { m |= 1ull << 52; e = (int)ex - 1075; }\n"
  "  const int s = e + sh;\n"
  "  if (ex == 0x7ffu || s > 9) return __double2ll_rn(__longlong_as_double((long long)bits) * sc);\n"
  "  u64 mag;\n"
  "  if (s >= 0) mag = m << s;\n"
  "  else if (s < -63) mag = 0ull;\n"
  "  else { const u32 r = (u32)(-s); const u64 q = m >> r, rem = m & ((1ull << r) - 1ull), half = 1ull << (r - 1u);\n"
  "         mag = q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull); }\n"
  "  return (bits >> 63) ? -(long long)mag : (long long)mag;\n"
  "}\n";

/* CTAs per SM of the register form at a block size: its shared accumulators are (block / 32) x 384 x 12
   bytes, 6 CTAs of 256 threads an SM */
static uint32_t register_ctas_per_sm(uint32_t block)
{
  return BATCH_CTAS_PER_SM * 256u / block;
}

/* The persistent form's additions: the queue loop's helpers. A slot's parameters are rewritten by copies
   between the kernel's uses of them; every thread passes a gpu-scope acquire fence after its CTA has seen the
   slot's new sequence number (read with an acquire load), so the scan's ordinary loads that follow do not
   see lines its SM's L1 kept from the slot's last use. */
static const char* PERSIST_PRELUDE =
  "__device__ __forceinline__ unsigned long long cql_cg64(const void* p) { unsigned long long v; asm volatile(\"ld.global.cg.u64 %0, [%1];\" : \"=l\"(v) : \"l\"(p)); return v; }\n"
  "__device__ __forceinline__ u64 cql_now() { u64 t; asm volatile(\"mov.u64 %0, %%globaltimer;\" : \"=l\"(t)); return t; }\n"
  "__device__ __forceinline__ u64 cql_acquire64(const void* p) { u64 v; asm volatile(\"ld.acquire.gpu.global.u64 %0, [%1];\" : \"=l\"(v) : \"l\"(p) : \"memory\"); return v; }\n"
  "__device__ __forceinline__ void cql_release_sys64(void* p, u64 v) { asm volatile(\"st.release.sys.global.u64 [%0], %1;\" :: \"l\"(p), \"l\"(v) : \"memory\"); }\n";

/* The persistent entry (cql_persist): every CTA waits for the next sequence number in the ring (thread 0
   polls, at most the idle limit, then the CTA returns; the stop word ~0 returns at once), builds the slot's launch in shared memory and runs
   the scan over its share of the table, adding its totals into the slot's accumulators with atomics (exact
   integer sums, so the order does not matter); the CTA that finishes last copies the answers into host
   memory, clears the accumulators and its ticket, and publishes the sequence number as done.
     p.buf[0]  ring: the sequence number of each slot (R u64, device; the host's copy of it lands after the
               slot's parameters)
     p.buf[1]  the slots' parameters (R x SB bytes, device): scales (256 B), a header (nq, need | sums << 32),
               thresholds at 512, literals, summed columns, shape starts - the ordinary launch's layout
     p.buf[2]  the slots' accumulators (R x NQ x 3 u64: count, low, high of the scaled sum)
     p.buf[3]  the slots' CTA tickets (R u32)
     p.buf[4]  answers (R x NQ x 3 u64, page-locked host memory)
     p.buf[5]  done words (R u64, page-locked host memory)
     p.buf[6 + c] the columns
   words: 0 rows, 2 R, 4 NQ, 6 SB, 8 idle limit (microseconds), 10 and 11 the first sequence number */
static const char* PERSIST_ENTRY =
  "extern \"C\" __global__ void __launch_bounds__(CQL_BLOCK, CQL_MIN_BLOCKS) cql_persist(CqlLaunch p)\n{\n"
  "  __shared__ CqlLaunch s_a; __shared__ u32 s_go, s_last;\n"
  "  const u64 rows = cql_word(p, 0); const u32 R = cql_word(p, 2), NQ = cql_word(p, 4), SB = cql_word(p, 6);\n"
  "  const u64 idle_ns = (u64)cql_word(p, 8) * 1000ull;\n"
  "  u64 seq = (u64)cql_word(p, 10) | ((u64)cql_word(p, 11) << 32);\n"
  "  const u64 off_qc = 512ull + (u64)NQ * 16ull * 32ull, off_qs = off_qc + (u64)NQ * 32ull * 8ull, off_begin = off_qs + (((u64)NQ * 4ull + 15ull) & ~15ull);\n"
  "  for (;; seq++)\n  {\n"
  "    const u32 slot = (u32)(seq % R);\n"
  "    if (threadIdx.x == 0)\n    {\n"
  "      const u64* ring = (const u64*)p.buf[0] + slot;\n"
  "      const u64 t0 = cql_now(); u32 go = 0u;\n"
  "      for (;;) { const u64 v = cql_acquire64(ring); if (v == seq) { go = 1u; break; } if (v == ~0ull || cql_now() - t0 > idle_ns) break; __nanosleep(256); }\n"
  "      s_go = go;\n"
  "      if (go)\n      {\n"
  "        const char* sp = (const char*)p.buf[1] + (u64)slot * SB;\n"
  "        const u64 nq = cql_cg64(sp + 256), needs = cql_cg64(sp + 264);\n"
  "        for (int i = 0; i < 16; i++) { s_a.buf[i] = p.buf[i]; s_a.bytes[i] = p.bytes[i]; }\n"
  "        s_a.buf[0] = (void*)sp; s_a.bytes[0] = 256ull;\n"
  "        s_a.buf[1] = (void*)(sp + 512); s_a.bytes[1] = off_qc - 512ull;\n"
  "        s_a.buf[2] = (void*)(sp + off_qc); s_a.bytes[2] = off_qs - off_qc;\n"
  "        s_a.buf[3] = (void*)(sp + off_qs); s_a.bytes[3] = (u64)NQ * 4ull;\n"
  "        s_a.buf[4] = (void*)(sp + off_begin); s_a.bytes[4] = (u64)SB - off_begin;\n"
  "        s_a.buf[5] = (void*)((u64*)p.buf[2] + (u64)slot * NQ * 3ull); s_a.bytes[5] = (u64)NQ * 24ull;\n"
  "        s_a.push[0] = rows; s_a.push[1] = nq; s_a.push[2] = 0ull; s_a.push[3] = needs;\n"
  "        for (int i = 4; i < 8; i++) s_a.push[i] = 0ull;\n"
  "      }\n"
  "    }\n"
  "    __syncthreads();\n"
  "    if (!s_go) return;\n"
  "    asm volatile(\"fence.acq_rel.gpu;\" ::: \"memory\");\n"
  "    cql_scan(s_a, blockIdx.x, gridDim.x);\n"
  "    __syncthreads();\n"
  "    if (threadIdx.x == 0) { __threadfence(); s_last = atomicAdd((u32*)p.buf[3] + slot, 1u) == gridDim.x - 1u; }\n"
  "    __syncthreads();\n"
  "    if (s_last)\n    {\n"
  "      __threadfence();\n"
  "      const u32 nq = (u32)s_a.push[1];\n"
  "      u64* acc = (u64*)s_a.buf[5];\n"
  "      u64* out = (u64*)p.buf[4] + (u64)slot * NQ * 3ull;\n"
  "      for (u32 i = threadIdx.x; i < nq * 3u; i += blockDim.x) { out[i] = cql_cg64(acc + i); acc[i] = 0ull; }\n"
  "      __threadfence_system();\n"
  "      __syncthreads();\n"
  "      if (threadIdx.x == 0) { ((u32*)p.buf[3])[slot] = 0u; __threadfence_system(); cql_release_sys64((u64*)p.buf[5] + slot, seq); }\n"
  "    }\n"
  "    __syncthreads();\n"
  "  }\n"
  "}\n";

/* the source of one launch: `shape_exprs` over `shapes` shapes, the register blocks of slot_type. persistent:
   the scan as a device function adding its totals into accumulators, entered by cql_main (one pass) and by
   the persistent queue loop cql_persist */
static char* batch_source(char** shape_exprs, const uint32_t* shape_sites, uint32_t shapes, const int* slot_type, const int* sum_cols,
                          uint32_t sum_col_count, uint32_t rows_per_thread, uint32_t block, int persistent)
{
  Buf b;
  memset(&b, 0, sizeof(b));
  bput(&b, "// cql: block=%u smem=%u per_sm=%u\n", block, (block / 32u) * CQL_BATCH_LAUNCH_QUERIES * 12u, register_ctas_per_sm(block));
  bput(&b, "%s", BATCH_PRELUDE);
  /* the persistent kernel's CTAs are all resident at once: at 4 rows a thread two of them an SM (the scan's
     registers fit 128 a thread), which the register bound keeps */
  if (persistent) bput(&b, "#define CQL_BLOCK %u\n#define CQL_MIN_BLOCKS %u\n%s", block, rows_per_thread <= 4 ? 2u : 1u, PERSIST_PRELUDE);
  for (uint32_t s = 0; s < shapes; s++) bput(&b, "#define CQL_SHAPE_%u(k) (%s)\n", s, shape_exprs[s]);
  if (persistent)
    bput(&b, "__device__ __forceinline__ void cql_scan(const CqlLaunch& a, const u32 cta, const u32 ctas)\n{\n");
  else
    bput(&b, "extern \"C\" __global__ void __launch_bounds__(%u) cql_main(CqlLaunch a)\n{\n  const u32 cta = blockIdx.x, ctas = gridDim.x;\n", block);
  bput(&b,
       "  const u64 rows = cql_word(a, 0); const u32 nq = cql_word(a, 2); const u32 q0 = cql_word(a, 4);\n"
       "  const u32 need = cql_word(a, 6), need_sum = cql_word(a, 7);   /* the columns this launch reads and sums */\n"
       "  (void)need_sum;\n"
       "  const double* col_scale = (const double*)a.buf[0];   /* 2^k per summed column, then k at [16 + column] */\n"
       "  const long long* col_shift = (const long long*)a.buf[0] + 16;\n"
       "  const Thr* thr = (const Thr*)a.buf[1];\n"
       "  const double* qconst = (const double*)a.buf[2];\n"
       "  const u32* qsum = (const u32*)a.buf[3];\n"
       "  const u32* shape_begin = (const u32*)a.buf[4];\n"
       "  u64* partials = (u64*)a.buf[5]; const u64 pcap = a.bytes[5] / 24ull;\n"
       "  extern __shared__ u64 s_acc[];   /* [warp][query] sums, then [warp][query] counts */\n"
       "  const u32 lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;\n"
       "  u32* s_cnt = (u32*)(s_acc + (u64)warps * nq);\n"
       "  for (u32 i = threadIdx.x; i < warps * nq; i += blockDim.x) { s_acc[i] = 0ull; s_cnt[i] = 0u; }\n"
       "  __syncthreads();\n"
       "  long long* acc = (long long*)s_acc + (u64)warp * nq; u32* cacc = s_cnt + (u64)warp * nq;\n");
  /* the columns' addresses in registers before the row loop (the persistent form's launch lives in shared memory) */
  for (int sl = 0; sl < CQLOPS_MAX_BINDINGS; sl++)
    if (slot_type[sl]) bput(&b, "  const void* const colp%d = a.buf[%d];\n", sl, 6 + sl);
  bput(&b,
       "  const u32 RPT = %uu;\n"
       "  const u64 groups = (rows + RPT - 1ull) / RPT; const u64 per_pass = (u64)ctas * blockDim.x;\n"
       "  for (u64 g0 = (u64)cta * blockDim.x; g0 < groups; g0 += per_pass)\n  {\n"
       "    const u64 row0 = (g0 + threadIdx.x) * RPT;\n"
       "    const u32 valid = row0 < rows ? (u32)min((u64)RPT, rows - row0) : 0u;\n"
       "    const u32 valid_mask = valid >= 32u ? 0xffffffffu : ((1u << valid) - 1u);\n",
       rows_per_thread);
  /* the register blocks */
  for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++)
  {
    int t = slot_type[s];
    if (!t) continue;
    int w = type_bytes(t);
    /* a column no query of the launch reads is not loaded (a grid-uniform branch) */
    bput(&b, "    %s r%d[%u];\n    if (!((need >> %d) & 1u)) { for (u32 v = 0; v < RPT; v++) r%d[v] = 0u; }\n", w == 8 ? "u64" : "u32", s,
         rows_per_thread, s, s);
    if (w == 8)
      bput(&b, "    else { for (u32 v = 0; v < RPT; v++) r%d[v] = v < valid ? ((const u64*)colp%d)[row0 + v] : 0ull; }\n", s, s);
    else if (w == 1)
      bput(&b, "    else { for (u32 v = 0; v < RPT; v++) r%d[v] = v < valid ? (u32)((const unsigned char*)colp%d)[row0 + v] : 0u; }\n", s, s);
    else
      bput(&b,
           "    else if (valid == RPT && (RPT & 3u) == 0u) { for (u32 v = 0; v < RPT; v += 4) { uint4 q = cql_ld4((const u32*)colp%d + row0 + v); r%d[v] = q.x; r%d[v + 1] = q.y; r%d[v + 2] = q.z; r%d[v + 3] = q.w; } }\n"
           "    else { for (u32 v = 0; v < RPT; v++) r%d[v] = v < valid ? ((const u32*)colp%d)[row0 + v] : 0u; }\n",
           s, s, s, s, s, s, s);
  }
  /* the order keys of the f64 columns, once per row (every query's comparisons read them) */
  for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++)
    if (slot_type[s] == CQLOPS_TYPE_F64) bput(&b, "    u64 kd%d[%u];\n    for (u32 v = 0; v < RPT; v++) kd%d[v] = cql_key(r%d[v]);\n", s, rows_per_thread, s, s);
  /* the summed columns as scaled integers, once per row */
  for (uint32_t i = 0; i < sum_col_count; i++)
  {
    int c = sum_cols[i];
    int t = slot_type[c];
    /* the value times 2^k as an integer: a shift for whole numbers, the bits of a float otherwise; FP64
       arithmetic only for 64-bit integers (the GPU's FP64 rate is a small fraction of its integer rate) */
    char expr[200];
    if (t == CQLOPS_TYPE_F64) snprintf(expr, sizeof(expr), "cql_fx64(r%d[v], sh, sc)", c);
    else if (t == CQLOPS_TYPE_F32) snprintf(expr, sizeof(expr), "cql_fx64((u64)__double_as_longlong((double)__uint_as_float(r%d[v])), sh, sc)", c);
    else if (t == CQLOPS_TYPE_I32)
      snprintf(expr, sizeof(expr), "(sh >= 0 ? (long long)(int)r%d[v] * (1ll << sh) : __double2ll_rn((double)(int)r%d[v] * sc))", c, c);
    else if (t == CQLOPS_TYPE_U64) snprintf(expr, sizeof(expr), "__double2ll_rn((double)r%d[v] * sc)", c);
    else if (t == CQLOPS_TYPE_I64) snprintf(expr, sizeof(expr), "__double2ll_rn(cql_i64d(r%d[v]) * sc)", c);
    else snprintf(expr, sizeof(expr), "(sh >= 0 ? (long long)((u64)r%d[v] << sh) : __double2ll_rn((double)r%d[v] * sc))", c, c);
    bput(&b, "    long long fx%d[%u];\n    if (!((need_sum >> %d) & 1u)) { for (u32 v = 0; v < RPT; v++) fx%d[v] = 0ll; }\n", c, rows_per_thread, c, c);
    bput(&b, "    else { const double sc = col_scale[%d]; const int sh = (int)col_shift[%d]; (void)sh; (void)sc;\n", c, c);
    bput(&b, "      for (u32 v = 0; v < RPT; v++) fx%d[v] = v < valid ? %s : 0ll; }\n", c, expr);
  }
  for (uint32_t s = 0; s < shapes; s++)
  {
    /* the query's thresholds into registers once, before its rows */
    char decls[BATCH_MAX_SITES * 40 + 1];
    size_t dn = 0;
    decls[0] = 0;
    for (uint32_t i = 0; i < shape_sites[s] && i < BATCH_MAX_SITES; i++)
      dn += (size_t)snprintf(decls + dn, sizeof(decls) - dn, "      const Thr T%u = TH[%u];\n", i, i);
    bput(&b,
         "    for (u32 q = shape_begin[%u]; q < shape_begin[%u]; q++)\n    {\n"
         "      const Thr* TH = thr + (u64)(q0 + q) * %uu; const double* QC = qconst + (u64)(q0 + q) * %uu;\n"
         "      (void)TH; (void)QC;\n"
         "%s"
         "      u32 m = 0u;\n"
         "#pragma unroll\n"
         "      for (u32 k = 0; k < RPT; k++) m |= ((CQL_SHAPE_%u(k)) ? 1u : 0u) << k;\n"
         "      m &= valid_mask;\n"
         "      const u32 cnt = __reduce_add_sync(0xffffffffu, (u32)__popc(m));\n"
         "      const u32 sc = qsum[q0 + q];\n"
         "      long long sv = 0ll;\n",
         s, s + 1, BATCH_MAX_SITES, BATCH_MAX_CONSTS, decls, s);
    for (uint32_t i = 0; i < sum_col_count; i++)
      bput(&b, "      if (sc == %du && m) {\n#pragma unroll\n        for (u32 k = 0; k < RPT; k++) if ((m >> k) & 1u) sv += fx%d[k];\n      }\n", sum_cols[i],
           sum_cols[i]);
    bput(&b,
         "      if (sc != 0xffffffffu) sv = cql_wsum64(sv);\n"
         "      if (lane == 0u) { cacc[q] += cnt; acc[q] += sv; }\n"
         "    }\n");
  }
  bput(&b,
       "  }\n"
       "  __syncthreads();\n"
       "  for (u32 q = threadIdx.x; q < nq; q += blockDim.x)\n  {\n"
       "    u64 c = 0ull, lo = 0ull, hi = 0ull;\n"
       "    for (u32 w = 0; w < warps; w++) { long long v = (long long)s_acc[(u64)w * nq + q]; c += s_cnt[(u64)w * nq + q];\n"
       "      u64 l2 = lo + (u64)v; hi += (u64)(v < 0 ? -1ll : 0ll) + (l2 < lo ? 1ull : 0ull); lo = l2; }\n"
       "%s"
       "  }\n"
       "}\n",
       persistent ? /* the CTA's 128-bit totals added into the accumulators: the low words with a carry into the high */
                    "    if (q < pcap && (c | lo | hi)) { if (c) atomicAdd(&partials[q * 3], c); const u64 old = atomicAdd(&partials[q * 3 + 1], lo);\n"
                    "      const u64 up = hi + ((old + lo < old) ? 1ull : 0ull); if (up) atomicAdd(&partials[q * 3 + 2], up); }\n"
                  : "    const u64 at = (u64)cta * nq + q;\n"
                    "    if (at < pcap) { partials[at * 3] = c; partials[at * 3 + 1] = lo; partials[at * 3 + 2] = hi; }\n");
  if (persistent)
    bput(&b, "extern \"C\" __global__ void __launch_bounds__(CQL_BLOCK) cql_main(CqlLaunch a) { cql_scan(a, blockIdx.x, gridDim.x); }\n%s",
         PERSIST_ENTRY);
  if (b.failed)
  {
    free(b.p);
    return NULL;
  }
  return b.p;
}

/* ---- the operator ---- */

static uint64_t fnv_str(const char* s)
{
  uint64_t h = 1469598103934665603ull;
  for (; *s; s++) h = (h ^ (unsigned char)*s) * 1099511628211ull;
  return h;
}

static CqlBuffer* pooled(const char* name, uint64_t size, uint32_t flags)
{
  return cqlcuda_buffer_alloc_pooled(name, (uint64_t)strlen(name), size ? size : 8, flags, NULL);
}

/* ---- the shared-memory tile form ---- */

/* A CTA stages a tile of rows of every loaded column (32-bit values as they are, f64 columns as order
   keys, 64-bit integers raw) and of every summed column (its fixed-point summands) in shared memory; its
   warps then take (query, part of the tile) items, each lane walking the part's rows 32 apart with the
   count and sum in registers, and a warp adds its totals to the CTA's accumulators once per item - not
   once per few rows as the register form does. */
typedef struct
{
  uint32_t tile;     /* rows per tile: 1024 or 512 */
  uint32_t per_sm;   /* resident CTAs per SM the shared memory allows (at most 8) */
  uint32_t smem;     /* dynamic shared memory per CTA */
  uint32_t n32, n64; /* 32-bit and 64-bit tiles */
} TiledLayout;

#define TILED_SHAPE_SLOTS 260   /* the query-to-shape table in shared memory (u32 entries) */

static TiledLayout tiled_layout(const int* slot_type, uint32_t sum_col_count)
{
  TiledLayout l;
  l.n32 = 0;
  l.n64 = sum_col_count;
  for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++)
    if (slot_type[s])
    {
      if (type_bytes(slot_type[s]) == 8) l.n64++;
      else l.n32++;
    }
  uint32_t per_row = 4 * l.n32 + 8 * l.n64;
  uint32_t fixed = 2u * CQL_BATCH_LAUNCH_QUERIES * 8u + (CQL_BATCH_LAUNCH_QUERIES + TILED_SHAPE_SLOTS) * 4u;
  l.tile = per_row * 1024u + fixed <= 72u * 1024u ? 1024u : 512u;
  l.smem = per_row * l.tile + fixed;
  uint32_t per_sm = (227u * 1024u) / (l.smem + 1024u);
  l.per_sm = per_sm > 8 ? 8 : (per_sm < 1 ? 1 : per_sm);
  return l;
}

static char* batch_source_tiled(char** shape_exprs, const uint32_t* shape_sites, uint32_t shapes, const int* slot_type, const int* sum_cols,
                                uint32_t sum_col_count)
{
  TiledLayout L = tiled_layout(slot_type, sum_col_count);
  const uint32_t per_thread = L.tile / QE_GPU_WORKGROUP_SIZE;   /* rows a thread stages: 4 or 2 */
  Buf b;
  memset(&b, 0, sizeof(b));
  bput(&b, "// cql: block=%u smem=%u per_sm=%u\n", QE_GPU_WORKGROUP_SIZE, L.smem, L.per_sm);
  bput(&b, "%s", BATCH_PRELUDE);
  bput(&b, "struct KeyBits { const u64* p; __device__ __forceinline__ u64 operator[](u32 i) const { const u64 k = p[i]; return (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k; } };\n");
  for (uint32_t s = 0; s < shapes; s++) bput(&b, "#define CQL_SHAPE_%u(k) (%s)\n", s, shape_exprs[s]);
  bput(&b,
       "extern \"C\" __global__ void __launch_bounds__(%u) cql_main(CqlLaunch a)\n{\n"
       "  const u32 TILE = %uu, PT = %uu;\n"
       "  const u64 rows = cql_word(a, 0); const u32 nq = cql_word(a, 2); const u32 q0 = cql_word(a, 4);\n"
       "  const u32 need = cql_word(a, 6), need_sum = cql_word(a, 7);   /* the columns this launch reads and sums */\n"
       "  const double* col_scale = (const double*)a.buf[0];   /* 2^k per summed column, then k at [16 + column] */\n"
       "  const long long* col_shift = (const long long*)a.buf[0] + 16;\n"
       "  const Thr* thr = (const Thr*)a.buf[1];\n"
       "  const double* qconst = (const double*)a.buf[2];\n"
       "  const u32* qsum = (const u32*)a.buf[3];\n"
       "  const u32* shape_begin = (const u32*)a.buf[4];\n"
       "  u64* partials = (u64*)a.buf[5]; const u64 pcap = a.bytes[5] / 24ull;\n"
       "  (void)col_scale; (void)col_shift; (void)need_sum;\n"
       "  extern __shared__ u64 s_mem[];\n"
       "  u64* s_cnt = s_mem; u64* s_sum = s_mem + %uu;\n"
       "  u32* s_shape = (u32*)(s_mem + 2u * %uu);\n"
       "  u64* t64 = s_mem + 2u * %uu + (%uu + 1u) / 2u;\n"
       "  u32* t32 = (u32*)(t64 + (u64)%uu * TILE);\n"
       "  const u32 lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;\n"
       "  for (u32 i = threadIdx.x; i < 2u * %uu; i += blockDim.x) s_mem[i] = 0ull;\n"
       "  for (u32 q = threadIdx.x; q < nq; q += blockDim.x) { u32 s = 0u; while (s + 1u < %uu && q >= shape_begin[s + 1u]) s++; s_shape[q] = s; }\n",
       QE_GPU_WORKGROUP_SIZE, L.tile, per_thread, CQL_BATCH_LAUNCH_QUERIES, CQL_BATCH_LAUNCH_QUERIES, CQL_BATCH_LAUNCH_QUERIES,
       CQL_BATCH_LAUNCH_QUERIES + TILED_SHAPE_SLOTS, L.n64, CQL_BATCH_LAUNCH_QUERIES, shapes + 1);
  /* the tiles: 64-bit ones first (f64 keys, raw 64-bit integers, then the summands), then 32-bit ones */
  uint32_t i64 = 0, i32 = 0;
  for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++)
  {
    int t = slot_type[s];
    if (!t) continue;
    if (type_bytes(t) == 8)
    {
      if (t == CQLOPS_TYPE_F64) bput(&b, "  u64* kd%d = t64 + %uu * TILE; const KeyBits r%d = { kd%d };\n", s, i64, s, s);
      else bput(&b, "  u64* r%d = t64 + %uu * TILE;\n", s, i64);
      i64++;
    }
    else
      bput(&b, "  u32* r%d = t32 + %uu * TILE;\n", s, i32++);
  }
  for (uint32_t i = 0; i < sum_col_count; i++) bput(&b, "  long long* fx%d = (long long*)(t64 + %uu * TILE);\n", sum_cols[i], i64++);
  bput(&b,
       "  const u32 parts = nq >= warps ? 1u : warps / nq;   /* few queries: each also split over the tile's rows */\n"
       "  const u32 items = nq * parts;\n"
       "  const u64 tiles = (rows + TILE - 1ull) / TILE;\n"
       "  const u32 i0 = threadIdx.x * PT;\n");
  /* each thread's PT consecutive rows of every needed column, fetched into registers one tile ahead: the
     next tile's loads are in flight while the warps evaluate this one */
  for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++)
    if (slot_type[s]) bput(&b, "  %s v%d[%u];\n", type_bytes(slot_type[s]) == 8 ? "u64" : "u32", s, per_thread);
  bput(&b, "  u64 tf = blockIdx.x;\n");
  char* fetch = NULL;
  {
    Buf f;
    memset(&f, 0, sizeof(f));
    bput(&f, "  {\n    const u64 fb = tf * TILE; const u32 fn = tf < tiles ? (u32)min((u64)TILE, rows - fb) : 0u;\n");
    for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++)
    {
      int t = slot_type[s];
      if (!t) continue;
      int w = type_bytes(t);
      bput(&f, "    if ((need >> %d) & 1u)\n    {\n", s);
      if (w == 8)
        bput(&f,
             "      if (fn == TILE) { for (u32 j = 0; j < PT; j += 2u) { uint4 x = cql_ld4((const u64*)a.buf[%d] + fb + i0 + j); v%d[j] = ((u64)x.y << 32) | x.x; v%d[j + 1] = ((u64)x.w << 32) | x.z; } }\n"
             "      else { for (u32 j = 0; j < PT; j++) v%d[j] = i0 + j < fn ? ((const u64*)a.buf[%d])[fb + i0 + j] : 0ull; }\n",
             6 + s, s, s, s, 6 + s);
      else if (w == 1)
        bput(&f, "      for (u32 j = 0; j < PT; j++) v%d[j] = i0 + j < fn ? (u32)((const unsigned char*)a.buf[%d])[fb + i0 + j] : 0u;\n", s, 6 + s);
      else if (per_thread == 4)
        bput(&f,
             "      if (fn == TILE) { uint4 x = cql_ld4((const u32*)a.buf[%d] + fb + i0); v%d[0] = x.x; v%d[1] = x.y; v%d[2] = x.z; v%d[3] = x.w; }\n"
             "      else { for (u32 j = 0; j < 4u; j++) v%d[j] = i0 + j < fn ? ((const u32*)a.buf[%d])[fb + i0 + j] : 0u; }\n",
             6 + s, s, s, s, s, s, 6 + s);
      else
        bput(&f, "      for (u32 j = 0; j < PT; j++) v%d[j] = i0 + j < fn ? ((const u32*)a.buf[%d])[fb + i0 + j] : 0u;\n", s, 6 + s);
      bput(&f, "    }\n");
    }
    bput(&f, "  }\n");
    if (f.failed)
    {
      free(f.p);
      b.failed = 1;
    }
    else
      fetch = f.p;
  }
  if (fetch) bput(&b, "%s", fetch);
  bput(&b,
       "  __syncthreads();\n"
       "  for (u64 t = blockIdx.x; t < tiles; t += gridDim.x)\n  {\n"
       "    const u64 base = t * TILE;\n"
       "    const u32 n = (u32)min((u64)TILE, rows - base);\n"
       "    (void)base;\n");
  /* staging: the fetched registers into the tiles (f64 columns as order keys, summed columns also as
     their fixed-point summands) */
  for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++)
  {
    int t = slot_type[s];
    if (!t) continue;
    int summed = 0;
    for (uint32_t i = 0; i < sum_col_count; i++)
      if (sum_cols[i] == s) summed = 1;
    bput(&b, "    if ((need >> %d) & 1u)\n    {\n", s);
    if (t == CQLOPS_TYPE_F64) bput(&b, "      for (u32 j = 0; j < PT; j++) kd%d[i0 + j] = cql_key(v%d[j]);\n", s, s);
    else bput(&b, "      for (u32 j = 0; j < PT; j++) r%d[i0 + j] = v%d[j];\n", s, s);
    if (summed)
    {
      char expr[220];
      if (t == CQLOPS_TYPE_F64) snprintf(expr, sizeof(expr), "cql_fx64(v%d[j], sh, sc)", s);
      else if (t == CQLOPS_TYPE_F32) snprintf(expr, sizeof(expr), "cql_fx64((u64)__double_as_longlong((double)__uint_as_float(v%d[j])), sh, sc)", s);
      else if (t == CQLOPS_TYPE_I32)
        snprintf(expr, sizeof(expr), "(sh >= 0 ? (long long)(int)v%d[j] * (1ll << sh) : __double2ll_rn((double)(int)v%d[j] * sc))", s, s);
      else if (t == CQLOPS_TYPE_U64) snprintf(expr, sizeof(expr), "__double2ll_rn((double)v%d[j] * sc)", s);
      else if (t == CQLOPS_TYPE_I64) snprintf(expr, sizeof(expr), "__double2ll_rn(cql_i64d(v%d[j]) * sc)", s);
      else snprintf(expr, sizeof(expr), "(sh >= 0 ? (long long)((u64)v%d[j] << sh) : __double2ll_rn((double)v%d[j] * sc))", s, s);
      bput(&b,
           "      if ((need_sum >> %d) & 1u) { const double sc = col_scale[%d]; const int sh = (int)col_shift[%d]; (void)sc; (void)sh;\n"
           "        for (u32 j = 0; j < PT; j++) fx%d[i0 + j] = i0 + j < n ? %s : 0ll; }\n",
           s, s, s, s, expr);
    }
    bput(&b, "    }\n");
  }
  bput(&b, "    __syncthreads();\n    tf = t + gridDim.x;\n");
  if (fetch) bput(&b, "%s", fetch);
  free(fetch);
  bput(&b,
       "    for (u32 it = warp; it < items; it += warps)\n    {\n"
       "      const u32 q = it / parts, part = it - q * parts;\n"
       "      const u32 span = (n + parts - 1u) / parts;\n"
       "      const u32 lo = min(n, part * span), hi = min(n, lo + span);\n"
       "      const Thr* TH = thr + (u64)(q0 + q) * %uu; const double* QC = qconst + (u64)(q0 + q) * %uu;\n"
       "      (void)TH; (void)QC;\n"
       "      const u32 sc = qsum[q0 + q];\n"
       "      const long long* fxp = ",
       BATCH_MAX_SITES, BATCH_MAX_CONSTS);
  for (uint32_t i = 0; i < sum_col_count; i++) bput(&b, "sc == %du ? fx%d : ", sum_cols[i], sum_cols[i]);
  bput(&b,
       "(const long long*)0;\n"
       "      (void)fxp;\n"
       "      u32 cnt = 0u; long long sv = 0ll;\n"
       "      switch (s_shape[q])\n      {\n");
  for (uint32_t s = 0; s < shapes; s++)
  {
    char decls[BATCH_MAX_SITES * 40 + 1];
    size_t dn = 0;
    decls[0] = 0;
    for (uint32_t i = 0; i < shape_sites[s] && i < BATCH_MAX_SITES; i++)
      dn += (size_t)snprintf(decls + dn, sizeof(decls) - dn, "        const Thr T%u = TH[%u];\n", i, i);
    bput(&b,
         "      case %uu:\n      {\n"
         "%s"
         "        if (!fxp) { for (u32 k = lo + lane; k < hi; k += 32u) cnt += (CQL_SHAPE_%u(k)) ? 1u : 0u; }\n"
         "        else { for (u32 k = lo + lane; k < hi; k += 32u) { const bool m = CQL_SHAPE_%u(k); cnt += m ? 1u : 0u; sv += m ? fxp[k] : 0ll; } }\n"
         "        break;\n      }\n",
         s, decls, s, s);
  }
  bput(&b,
       "      default: break;\n"
       "      }\n"
       "      cnt = __reduce_add_sync(0xffffffffu, cnt);\n"
       "      if (fxp) sv = cql_wsum64(sv);\n"
       "      if (lane == 0u) { atomicAdd(&s_cnt[q], (u64)cnt); if (sv) atomicAdd(&s_sum[q], (u64)sv); }\n"
       "    }\n"
       "    __syncthreads();\n"
       "  }\n"
       "  for (u32 q = threadIdx.x; q < nq; q += blockDim.x)\n  {\n"
       "    const long long v = (long long)s_sum[q];\n"
       "    const u64 at = (u64)blockIdx.x * nq + q;\n"
       "    if (at < pcap) { partials[at * 3] = s_cnt[q]; partials[at * 3 + 1] = (u64)v; partials[at * 3 + 2] = v < 0 ? ~0ull : 0ull; }\n"
       "  }\n}\n");
  if (b.failed)
  {
    free(b.p);
    return NULL;
  }
  return b.p;
}

/* ---- the cube form: group once, answer many ---- */

/* Queries whose WHERE reads only whole-number columns of small range are answered from a dense table of
   the rows: for every combination of those columns' values (a cell) the count of rows and the
   fixed-point sums of the summed columns, built in one pass over the table (shared-memory tables per CTA,
   then 128-bit totals in global memory). A query then tests its predicate on each cell's values - the
   values of the rows in that cell, so the test is the rows' test - and adds up the cells that pass.
   Counts are exact and the sums are the same integers the scan adds, so the results are the scan's;
   the table costs one pass whatever the number of queries, and a query costs a pass over the cells. */
#define CUBE_MAX 8
#define CUBE_MAX_DIMS 4
#define CUBE_MAX_CELLS 65536u
#define CUBE_SMEM_BYTES (200u * 1024u)
#define CUBE_THREADS 1024u
#define CUBE_MIN_QUERIES 6u

typedef struct
{
  uint32_t dims;
  int slot[CUBE_MAX_DIMS];
  uint32_t min[CUBE_MAX_DIMS];      /* the column's smallest value (bits of the i32 for I32 columns) */
  uint32_t radix[CUBE_MAX_DIMS];
  uint32_t stride[CUBE_MAX_DIMS];
  int is_signed[CUBE_MAX_DIMS];
  uint32_t cells;
  uint32_t mask;                    /* the slots */
  uint32_t nsum;
  int sum_slot[CQLOPS_MAX_BINDINGS];
  uint64_t word_off;                /* first word of the cube's global table: counts, then (lo, hi) sums */
  uint32_t pass;                    /* the table pass that builds it */
  uint32_t smem_off;                /* bytes into its pass's shared tables: u32 counts, then 128-bit sums [sum][cell] */
} Cube;

typedef struct
{
  uint32_t cubes;
  Cube cube[CUBE_MAX];
  uint64_t words;
  uint32_t passes;                  /* table passes: each builds the cubes whose shared tables fit together */
  uint32_t smem[CUBE_MAX];          /* one copy of a pass's shared tables */
  uint32_t copies[CUBE_MAX];        /* copies of them per CTA (warps spread over them) */
} CubePlan;

static uint32_t cube_smem(const Cube* c)
{
  return ((c->cells * 4u + 7u) & ~7u) + c->cells * c->nsum * 16u;
}

/* whether column `slot` can be a dimension: a whole-number column of at most 65536 values */
static int cube_dim_ok(const CqlColumn* columns, uint32_t column_count, int slot, int load_type)
{
  if (slot < 0 || (uint32_t)slot >= column_count) return 0;
  const CqlColumn* c = &columns[slot];
  if (!(load_type == CQLOPS_TYPE_U32 || load_type == CQLOPS_TYPE_I32) || c->type != (uint32_t)load_type || !c->has_range) return 0;
  if (!(c->zone_max >= c->zone_min) || c->zone_max - c->zone_min > 65535.0) return 0;
  if (load_type == CQLOPS_TYPE_U32 && (c->zone_min < 0.0 || c->zone_max > 4294967295.0)) return 0;
  if (load_type == CQLOPS_TYPE_I32 && (c->zone_min < -2147483648.0 || c->zone_max > 2147483647.0)) return 0;
  return 1;
}

/* Assigns shapes to cubes: each eligible shape's column set, merged into a cube over a superset when one
   exists. When the shared tables do not fit, the largest cube's column set is excluded and the plan made
   again (its shapes may then join other cubes or get their own; a shape over an excluded set goes to the
   scan). cube_of[s] = -1 for a shape the scan answers. */
static void cube_assign(uint32_t shapes, const uint32_t* shape_mask, const uint32_t* shape_sums, const int* eligible,
                        const uint32_t* excluded, uint32_t excluded_count, const CqlColumn* columns, CubePlan* plan, int* cube_of)
{
  memset(plan, 0, sizeof(*plan));
  uint32_t order[BATCH_MAX_SHAPES];
  uint32_t n = 0;
  for (uint32_t s = 0; s < shapes; s++)
  {
    cube_of[s] = -1;
    int out = !eligible[s];
    for (uint32_t e = 0; !out && e < excluded_count; e++) out = shape_mask[s] == excluded[e];
    if (!out) order[n++] = s;
  }
  for (uint32_t i = 1; i < n; i++)
    for (uint32_t j = i; j > 0 && __builtin_popcount(shape_mask[order[j]]) > __builtin_popcount(shape_mask[order[j - 1]]); j--)
    {
      uint32_t t = order[j];
      order[j] = order[j - 1];
      order[j - 1] = t;
    }
  for (uint32_t i = 0; i < n; i++)
  {
    uint32_t s = order[i], m = shape_mask[s];
    int chosen = -1;
    for (uint32_t c = 0; c < plan->cubes && chosen < 0; c++)
      if ((plan->cube[c].mask & m) == m) chosen = (int)c;
    if (chosen < 0 && plan->cubes < CUBE_MAX)
    {
      Cube* c = &plan->cube[plan->cubes];
      memset(c, 0, sizeof(*c));
      c->mask = m;
      for (int d = 0; d < CQLOPS_MAX_BINDINGS; d++)
        if ((m >> d) & 1u)
        {
          c->slot[c->dims] = d;
          c->is_signed[c->dims] = columns[d].type == CQLOPS_TYPE_I32;
          c->min[c->dims] = c->is_signed[c->dims] ? (uint32_t)(int32_t)columns[d].zone_min : (uint32_t)columns[d].zone_min;
          c->radix[c->dims] = (uint32_t)(columns[d].zone_max - columns[d].zone_min) + 1u;
          c->dims++;
        }
      /* row-major strides: the last dimension varies fastest */
      uint32_t stride = 1;
      for (int d = (int)c->dims - 1; d >= 0; d--)
      {
        c->stride[d] = stride;
        stride *= c->radix[d];
      }
      c->cells = stride;
      chosen = (int)plan->cubes++;
    }
    cube_of[s] = chosen;
  }
  /* summed columns of each cube: those its shapes' queries sum */
  for (uint32_t s = 0; s < shapes; s++)
  {
    if (cube_of[s] < 0) continue;
    Cube* c = &plan->cube[cube_of[s]];
    for (int col = 0; col < CQLOPS_MAX_BINDINGS; col++)
    {
      if (!((shape_sums[s] >> col) & 1u)) continue;
      uint32_t j = 0;
      while (j < c->nsum && c->sum_slot[j] != col) j++;
      if (j == c->nsum) c->sum_slot[c->nsum++] = col;
    }
  }
  /* global tables one after another; passes by first fit, largest cube first */
  uint64_t words = 0;
  for (uint32_t c = 0; c < plan->cubes; c++)
  {
    plan->cube[c].word_off = words;
    words += (uint64_t)plan->cube[c].cells * (1u + 2u * plan->cube[c].nsum);
  }
  plan->words = words;
  uint32_t by_size[CUBE_MAX];
  for (uint32_t c = 0; c < plan->cubes; c++) by_size[c] = c;
  for (uint32_t i = 1; i < plan->cubes; i++)
    for (uint32_t j = i; j > 0 && cube_smem(&plan->cube[by_size[j]]) > cube_smem(&plan->cube[by_size[j - 1]]); j--)
    {
      uint32_t t = by_size[j];
      by_size[j] = by_size[j - 1];
      by_size[j - 1] = t;
    }
  plan->passes = 0;
  for (uint32_t i = 0; i < plan->cubes; i++)
  {
    Cube* cu = &plan->cube[by_size[i]];
    uint32_t b = cube_smem(cu), p = 0;
    while (p < plan->passes && plan->smem[p] + b > CUBE_SMEM_BYTES) p++;
    if (p == plan->passes) plan->smem[plan->passes++] = 0;
    cu->pass = p;
    cu->smem_off = plan->smem[p];
    plan->smem[p] += b;
  }
  for (uint32_t p = 0; p < plan->passes; p++)
  {
    uint32_t copies = plan->smem[p] ? CUBE_SMEM_BYTES / plan->smem[p] : 1;
    plan->copies[p] = copies > 32 ? 32 : (copies < 1 ? 1 : copies);
  }
}

static void cube_plan(uint32_t shapes, const uint32_t* shape_mask, const int* shape_types, const uint32_t* shape_sums,
                      const CqlColumn* columns, uint32_t column_count, CubePlan* plan, int* cube_of)
{
  /* eligible: at most 4 whole-number columns of small range, at most CUBE_MAX_CELLS combinations */
  int eligible[BATCH_MAX_SHAPES];
  for (uint32_t s = 0; s < shapes; s++)
  {
    uint32_t m = shape_mask[s];
    int ok = __builtin_popcount(m) <= CUBE_MAX_DIMS;
    double cells = 1.0;
    for (int d = 0; ok && d < CQLOPS_MAX_BINDINGS; d++)
      if ((m >> d) & 1u)
      {
        ok = cube_dim_ok(columns, column_count, d, shape_types[s * CQLOPS_MAX_BINDINGS + d]);
        if (ok) cells *= columns[d].zone_max - columns[d].zone_min + 1.0;
      }
    eligible[s] = ok && cells <= (double)CUBE_MAX_CELLS;
  }
  /* a cube whose shared table alone is too large is not built: its column set is excluded and the
     shapes planned again (they may fit smaller cubes) */
  uint32_t excluded[BATCH_MAX_SHAPES];
  uint32_t excluded_count = 0;
  for (;;)
  {
    cube_assign(shapes, shape_mask, shape_sums, eligible, excluded, excluded_count, columns, plan, cube_of);
    int too_large = -1;
    for (uint32_t c = 0; c < plan->cubes && too_large < 0; c++)
      if (cube_smem(&plan->cube[c]) > CUBE_SMEM_BYTES) too_large = (int)c;
    if (too_large < 0) break;
    excluded[excluded_count++] = plan->cube[too_large].mask;
  }
}

/* the summand of slot `c` of type t in the kernels' fixed point, from v (the loaded word(s)) */
static void fx_expr(char* out, size_t cap, int t, const char* v)
{
  if (t == CQLOPS_TYPE_F64) snprintf(out, cap, "cql_fx64(%s, sh, sc)", v);
  else if (t == CQLOPS_TYPE_F32) snprintf(out, cap, "cql_fx64((u64)__double_as_longlong((double)__uint_as_float(%s)), sh, sc)", v);
  else if (t == CQLOPS_TYPE_I32) snprintf(out, cap, "(sh >= 0 ? (long long)(int)%s * (1ll << sh) : __double2ll_rn((double)(int)%s * sc))", v, v);
  else if (t == CQLOPS_TYPE_U64) snprintf(out, cap, "__double2ll_rn((double)%s * sc)", v);
  else if (t == CQLOPS_TYPE_I64) snprintf(out, cap, "__double2ll_rn(cql_i64d(%s) * sc)", v);
  else snprintf(out, cap, "(sh >= 0 ? (long long)((u64)%s << sh) : __double2ll_rn((double)%s * sc))", v, v);
}

/* The table pass: bindings 0 the scales, 1 the global tables (zeroed), 2 an error word, 6.. the columns;
   words 0 rows, 2 the summed columns this launch needs. */
static char* cube_build_source(const CubePlan* P, uint32_t pass, const int* slot_type)
{
  Buf b;
  memset(&b, 0, sizeof(b));
  const uint32_t SMEM = P->smem[pass], COPIES = P->copies[pass];
  uint32_t load = 0;   /* the columns the pass reads: dimensions and summed columns */
  for (uint32_t c = 0; c < P->cubes; c++)
  {
    if (P->cube[c].pass != pass) continue;
    load |= P->cube[c].mask;
    for (uint32_t j = 0; j < P->cube[c].nsum; j++) load |= 1u << P->cube[c].sum_slot[j];
  }
  bput(&b, "// cql: block=%u smem=%u per_sm=1\n", CUBE_THREADS, SMEM * COPIES);
  bput(&b, "%s", BATCH_PRELUDE);
  bput(&b,
       "extern \"C\" __global__ void __launch_bounds__(%u) cql_main(CqlLaunch a)\n{\n"
       "  const u64 rows = cql_word(a, 0); const u32 need_sum = cql_word(a, 2); (void)need_sum;\n"
       "  const u32 cube_need = cql_word(a, 4), load_need = cql_word(a, 6); (void)cube_need; (void)load_need;   /* the cubes this batch asks for, their columns */\n"
       "  const double* col_scale = (const double*)a.buf[0]; const long long* col_shift = (const long long*)a.buf[0] + 16;\n"
       "  (void)col_scale; (void)col_shift;\n"
       "  u64* g = (u64*)a.buf[1]; u32* err = (u32*)a.buf[2];\n"
       "  extern __shared__ u64 s_mem[];\n"
       "  for (u32 i = threadIdx.x; i < %uu; i += blockDim.x) s_mem[i] = 0ull;\n"
       "  __syncthreads();\n"
       "  unsigned char* tab = (unsigned char*)s_mem + ((threadIdx.x >> 5) %% %uu) * %uu;   /* this warp's copy */\n"
       "  u32 bad = 0u;\n"
       "  const u64 per_pass = (u64)gridDim.x * blockDim.x * 4ull;\n"
       "  for (u64 row0 = ((u64)blockIdx.x * blockDim.x + threadIdx.x) * 4ull; row0 < rows; row0 += per_pass)\n  {\n"
       "    const u32 valid = (u32)min((u64)4, rows - row0);\n",
       CUBE_THREADS, SMEM * COPIES / 8u, COPIES, SMEM);
  for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++)
  {
    if (!((load >> s) & 1u)) continue;
    int t = slot_type[s];
    if (type_bytes(t) == 8)
      bput(&b,
           "    u64 v%d[4];\n"
           "    if (!((load_need >> %d) & 1u)) { for (u32 j = 0; j < 4u; j++) v%d[j] = 0ull; }\n"
           "    else if (valid == 4u) { uint4 x = cql_ld4((const u64*)a.buf[%d] + row0); uint4 y = cql_ld4((const u64*)a.buf[%d] + row0 + 2);\n"
           "      v%d[0] = ((u64)x.y << 32) | x.x; v%d[1] = ((u64)x.w << 32) | x.z; v%d[2] = ((u64)y.y << 32) | y.x; v%d[3] = ((u64)y.w << 32) | y.z; }\n"
           "    else { for (u32 j = 0; j < 4u; j++) v%d[j] = j < valid ? ((const u64*)a.buf[%d])[row0 + j] : 0ull; }\n",
           s, s, s, 6 + s, 6 + s, s, s, s, s, s, 6 + s);
    else if (type_bytes(t) == 1)
      bput(&b, "    u32 v%d[4];\n    for (u32 j = 0; j < 4u; j++) v%d[j] = j < valid && ((load_need >> %d) & 1u) ? (u32)((const unsigned char*)a.buf[%d])[row0 + j] : 0u;\n",
           s, s, s, 6 + s);
    else
      bput(&b,
           "    u32 v%d[4];\n"
           "    if (!((load_need >> %d) & 1u)) { for (u32 j = 0; j < 4u; j++) v%d[j] = 0u; }\n"
           "    else if (valid == 4u) { uint4 x = cql_ld4((const u32*)a.buf[%d] + row0); v%d[0] = x.x; v%d[1] = x.y; v%d[2] = x.z; v%d[3] = x.w; }\n"
           "    else { for (u32 j = 0; j < 4u; j++) v%d[j] = j < valid ? ((const u32*)a.buf[%d])[row0 + j] : 0u; }\n",
           s, s, s, 6 + s, s, s, s, s, s, 6 + s);
  }
  /* the summands, once per row */
  uint32_t summed = 0;
  for (uint32_t c = 0; c < P->cubes; c++)
    if (P->cube[c].pass == pass)
      for (uint32_t j = 0; j < P->cube[c].nsum; j++) summed |= 1u << P->cube[c].sum_slot[j];
  for (int s = 0; s < CQLOPS_MAX_BINDINGS; s++)
  {
    if (!((summed >> s) & 1u)) continue;
    if (slot_type[s] == CQLOPS_TYPE_U32 || slot_type[s] == CQLOPS_TYPE_I32) continue;   /* whole numbers: their raw sum is kept */
    char vj[16], ex[220];
    snprintf(vj, sizeof(vj), "v%d[j]", s);
    fx_expr(ex, sizeof(ex), slot_type[s], vj);
    bput(&b,
         "    long long fx%d[4];\n"
         "    if ((need_sum >> %d) & 1u) { const double sc = col_scale[%d]; const int sh = (int)col_shift[%d]; (void)sc; (void)sh;\n"
         "      for (u32 j = 0; j < 4u; j++) fx%d[j] = j < valid ? %s : 0ll; }\n"
         "    else { for (u32 j = 0; j < 4u; j++) fx%d[j] = 0ll; }\n",
         s, s, s, s, s, ex, s);
  }
  bput(&b, "    for (u32 j = 0; j < valid; j++)\n    {\n");
  for (uint32_t c = 0; c < P->cubes; c++)
  {
    const Cube* cu = &P->cube[c];
    if (cu->pass != pass) continue;
    bput(&b, "      if ((cube_need >> %uu) & 1u)\n      {\n        u32 cell = 0u; bool in = true;\n", c);
    for (uint32_t d = 0; d < cu->dims; d++)
    {
      if (cu->is_signed[d]) bput(&b, "        { const u32 x = (u32)((int)v%d[j] - (int)%du); in = in && x < %uu; cell += x * %uu; }\n", cu->slot[d], cu->min[d], cu->radix[d], cu->stride[d]);
      else bput(&b, "        { const u32 x = v%d[j] - %uu; in = in && x < %uu; cell += x * %uu; }\n", cu->slot[d], cu->min[d], cu->radix[d], cu->stride[d]);
    }
    bput(&b,
         "        if (!in) bad = 1u;\n"
         "        else\n        {\n"
         "          atomicAdd((u32*)(tab + %uu) + cell, 1u);\n",
         cu->smem_off);
    uint32_t sums_at = cu->smem_off + ((cu->cells * 4u + 7u) & ~7u);
    /* a cell's sum is a 128-bit (lo, hi) pair: the low word by atomic add, the high word when the add
       carried or the summand is negative. A whole-number column adds its raw value into a 64-bit (lo, hi)
       pair of 32-bit words instead (one 32-bit atomic a row), scaled by 2^k when the tables are folded:
       the same integer as the sum of the scaled summands */
    for (uint32_t jj = 0; jj < cu->nsum; jj++)
    {
      int sl = cu->sum_slot[jj], t = slot_type[sl];
      if (t == CQLOPS_TYPE_U32 || t == CQLOPS_TYPE_I32)
        bput(&b,
             "          if (((need_sum >> %d) & 1u) && v%d[j]) { u32* w = (u32*)(tab + %uu) + 4u * (%uu + cell); const u32 v = v%d[j]; const u32 old = atomicAdd(&w[0], v);\n"
             "            const u32 h = (%s ? 0xffffffffu : 0u) + (old + v < old ? 1u : 0u); if (h) atomicAdd(&w[1], h); }\n",
             sl, sl, sums_at, jj * cu->cells, sl, t == CQLOPS_TYPE_I32 ? "(int)v < 0" : "false");
      else
        bput(&b,
             "          if (fx%d[j]) { u64* w = (u64*)(tab + %uu) + 2u * (%uu + cell); const u64 v = (u64)fx%d[j]; const u64 old = atomicAdd(&w[0], v);\n"
             "            const u64 h = (fx%d[j] < 0 ? ~0ull : 0ull) + (old + v < old ? 1ull : 0ull); if (h) atomicAdd(&w[1], h); }\n",
             sl, sums_at, jj * cu->cells, sl, sl);
    }
    bput(&b, "        }\n      }\n");
  }
  bput(&b, "    }\n  }\n  if (bad) atomicOr(err, 1u);\n  __syncthreads();\n");
  /* the copies folded into the global tables: counts added, sums as 128-bit totals */
  for (uint32_t c = 0; c < P->cubes; c++)
  {
    const Cube* cu = &P->cube[c];
    if (cu->pass != pass) continue;
    uint32_t sums_at = cu->smem_off + ((cu->cells * 4u + 7u) & ~7u);
    bput(&b,
         "  for (u32 cell = threadIdx.x; cell < %uu; cell += blockDim.x)\n  {\n"
         "    u64 n = 0ull;\n"
         "    for (u32 k = 0; k < %uu; k++) n += ((const u32*)((const unsigned char*)s_mem + k * %uu + %uu))[cell];\n"
         "    if (n) atomicAdd(&g[%lluull + cell], n);\n",
         cu->cells, COPIES, SMEM, cu->smem_off, (unsigned long long)cu->word_off);
    for (uint32_t jj = 0; jj < cu->nsum; jj++)
    {
      int sl = cu->sum_slot[jj], t = slot_type[sl];
      if (t == CQLOPS_TYPE_U32 || t == CQLOPS_TYPE_I32)
        /* the raw 64-bit sum over the copies, then times 2^k as a 128-bit pair (k >= 0 for columns of this
           range; otherwise the queries go back to the scan) */
        bput(&b,
             "    {\n      long long tot = 0;\n"
             "      for (u32 k = 0; k < %uu; k++) { const u32* v = (const u32*)((const unsigned char*)s_mem + k * %uu + %uu) + 4u * (%uu + cell);\n"
             "        tot += (long long)(((u64)v[1] << 32) | v[0]); }\n"
             "      const int sh = (int)col_shift[%d];\n"
             "      if (sh < 0 || sh > 62) { if (tot) atomicOr(err, 2u); }\n"
             "      else if (tot) { const u64 lo = (u64)tot << sh; const u64 hi = sh ? (u64)(tot >> (64 - sh)) : (tot < 0 ? ~0ull : 0ull);\n"
             "        u64* w = &g[%lluull + 2ull * ((u64)%uu + cell)]; const u64 old = atomicAdd(&w[0], lo);\n"
             "        const u64 carry = (old + lo < old) ? 1ull : 0ull; if (hi + carry) atomicAdd(&w[1], hi + carry); }\n"
             "    }\n",
             COPIES, SMEM, sums_at, jj * cu->cells, sl, (unsigned long long)(cu->word_off + cu->cells), jj * cu->cells);
      else
        bput(&b,
             "    {\n      u64 lo = 0ull, hi = 0ull;\n"
             "      for (u32 k = 0; k < %uu; k++) { const u64* v = (const u64*)((const unsigned char*)s_mem + k * %uu + %uu) + 2u * (%uu + cell);\n"
             "        const u64 l2 = lo + v[0]; hi += v[1] + (l2 < lo ? 1ull : 0ull); lo = l2; }\n"
             "      if (lo | hi) { u64* w = &g[%lluull + 2ull * ((u64)%uu + cell)]; const u64 old = atomicAdd(&w[0], lo);\n"
             "        const u64 carry = (old + lo < old) ? 1ull : 0ull; if (hi + carry) atomicAdd(&w[1], hi + carry); }\n"
             "    }\n",
             COPIES, SMEM, sums_at, jj * cu->cells, (unsigned long long)(cu->word_off + cu->cells), jj * cu->cells);
    }
    bput(&b, "  }\n");
  }
  bput(&b, "}\n");
  if (b.failed)
  {
    free(b.p);
    return NULL;
  }
  return b.p;
}

/* The answers: one CTA per query; bindings 1 the global tables, 3 thresholds, 4 literals, 5 per query
   (shape | cube << 8 | (summed column's index in the cube + 1) << 16), 6 out (count, lo, hi) per query;
   word 0 queries. */
static char* cube_answer_source(const CubePlan* P, char** shape_exprs, const uint32_t* shape_sites, uint32_t shapes, const int* cube_of)
{
  Buf b;
  memset(&b, 0, sizeof(b));
  bput(&b, "// cql: block=256 smem=0 per_sm=8\n");
  bput(&b, "%s", BATCH_PRELUDE);
  bput(&b, "struct CubeDim { u32 min, radix, stride; __device__ __forceinline__ u32 operator[](u32 cell) const { return min + (cell / stride) %% radix; } };\n");
  for (uint32_t s = 0; s < shapes; s++)
    if (cube_of[s] >= 0) bput(&b, "#define CQL_SHAPE_%u(k) (%s)\n", s, shape_exprs[s]);
  bput(&b,
       "extern \"C\" __global__ void __launch_bounds__(256) cql_main(CqlLaunch a)\n{\n"
       "  const u32 nq = cql_word(a, 0);\n"
       "  const u64* g = (const u64*)a.buf[1];\n"
       "  const Thr* thr = (const Thr*)a.buf[3]; const double* qconst = (const double*)a.buf[4];\n"
       "  const u32* meta = (const u32*)a.buf[5]; u64* out = (u64*)a.buf[6];\n"
       "  __shared__ u64 s_red[3 * 8];\n"
       "  for (u32 q = blockIdx.x; q < nq; q += gridDim.x)\n  {\n"
       "    const u32 m = meta[q]; const u32 shape = m & 0xffu, cube = (m >> 8) & 0xffu; const int sj = (int)(m >> 16) - 1;\n"
       "    const Thr* TH = thr + (u64)q * %uu; const double* QC = qconst + (u64)q * %uu; (void)TH; (void)QC;\n"
       "    u64 c = 0ull, lo = 0ull, hi = 0ull;\n"
       "    switch (cube)\n    {\n",
       BATCH_MAX_SITES, BATCH_MAX_CONSTS);
  for (uint32_t c = 0; c < P->cubes; c++)
  {
    const Cube* cu = &P->cube[c];
    bput(&b, "    case %uu:\n    {\n", c);
    for (uint32_t d = 0; d < cu->dims; d++)
      bput(&b, "      const CubeDim r%d = { %uu, %uu, %uu };\n", cu->slot[d], cu->min[d], cu->radix[d], cu->stride[d]);
    bput(&b,
         "      const u64* cnt = g + %lluull; const u64* sums = g + %lluull; (void)sums;\n"
         "      const u32 cells = %uu;\n"
         "      switch (shape)\n      {\n",
         (unsigned long long)cu->word_off, (unsigned long long)(cu->word_off + cu->cells), cu->cells);
    for (uint32_t s = 0; s < shapes; s++)
    {
      if (cube_of[s] != (int)c) continue;
      char decls[BATCH_MAX_SITES * 40 + 1];
      size_t dn = 0;
      decls[0] = 0;
      for (uint32_t i = 0; i < shape_sites[s] && i < BATCH_MAX_SITES; i++)
        dn += (size_t)snprintf(decls + dn, sizeof(decls) - dn, "        const Thr T%u = TH[%u];\n", i, i);
      bput(&b,
           "      case %uu:\n      {\n"
           "%s"
           "        for (u32 k = threadIdx.x; k < cells; k += blockDim.x)\n"
           "          if (CQL_SHAPE_%u(k)) { c += cnt[k]; if (sj >= 0) { const u64* w = sums + 2ull * ((u64)sj * cells + k); const u64 l2 = lo + w[0]; hi += w[1] + (l2 < lo ? 1ull : 0ull); lo = l2; } }\n"
           "        break;\n      }\n",
           s, decls, s);
    }
    bput(&b, "      default: break;\n      }\n      break;\n    }\n");
  }
  bput(&b,
       "    default: break;\n    }\n"
       "    for (int o = 16; o > 0; o >>= 1)\n    {\n"
       "      const u64 c2 = __shfl_xor_sync(0xffffffffu, c, o), l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);\n"
       "      const u64 s = lo + l2; hi += h2 + (s < lo ? 1ull : 0ull); lo = s; c += c2;\n"
       "    }\n"
       "    if ((threadIdx.x & 31u) == 0u) { s_red[(threadIdx.x >> 5) * 3] = c; s_red[(threadIdx.x >> 5) * 3 + 1] = lo; s_red[(threadIdx.x >> 5) * 3 + 2] = hi; }\n"
       "    __syncthreads();\n"
       "    if (threadIdx.x == 0u)\n    {\n"
       "      u64 tc = 0ull, tl = 0ull, th = 0ull;\n"
       "      for (u32 w = 0; w < blockDim.x / 32u; w++) { const u64 s = tl + s_red[w * 3 + 1]; th += s_red[w * 3 + 2] + (s < tl ? 1ull : 0ull); tl = s; tc += s_red[w * 3]; }\n"
       "      out[(u64)q * 3] = tc; out[(u64)q * 3 + 1] = tl; out[(u64)q * 3 + 2] = th;\n"
       "    }\n"
       "    __syncthreads();\n"
       "  }\n}\n");
  if (b.failed)
  {
    free(b.p);
    return NULL;
  }
  return b.p;
}

/* the source of one launch in the form rows_per_thread asks for */
static char* launch_source(char** shape_exprs, const uint32_t* shape_sites, uint32_t shapes, const int* slot_type, const int* sum_cols,
                           uint32_t sum_col_count, uint32_t rows_per_thread, uint32_t block, int persistent)
{
  if (!rows_per_thread) return batch_source_tiled(shape_exprs, shape_sites, shapes, slot_type, sum_cols, sum_col_count);
  return batch_source(shape_exprs, shape_sites, shapes, slot_type, sum_cols, sum_col_count, rows_per_thread, block, persistent);
}

/* ---- the shape catalog ---- */

struct CqlBatchCatalog
{
  pthread_mutex_t lock;
  uint32_t shapes;
  uint64_t keys[CQL_BATCH_CATALOG_SHAPES];
  char* exprs[CQL_BATCH_CATALOG_SHAPES];
  uint32_t sites[CQL_BATCH_CATALOG_SHAPES];
  uint32_t masks[CQL_BATCH_CATALOG_SHAPES];                       /* the columns each shape reads */
  int types[CQL_BATCH_CATALOG_SHAPES * CQLOPS_MAX_BINDINGS];      /* and as what */
  uint32_t sums[CQL_BATCH_CATALOG_SHAPES];                        /* the columns its queries have summed */
  int slot_type[CQLOPS_MAX_BINDINGS];
  uint32_t sum_mask;     /* the columns any batch summed */
  uint64_t version;      /* bumped when a shape, a column type or a summed column is added */
};

CqlBatchCatalog* cqlops_batch_catalog_create(void)
{
  CqlBatchCatalog* c = (CqlBatchCatalog*)calloc(1, sizeof(CqlBatchCatalog));
  if (c) pthread_mutex_init(&c->lock, NULL);
  return c;
}

void cqlops_batch_catalog_destroy(CqlBatchCatalog* c)
{
  if (!c) return;
  for (uint32_t s = 0; s < c->shapes; s++) free(c->exprs[s]);
  pthread_mutex_destroy(&c->lock);
  free(c);
}

uint32_t cqlops_batch_catalog_shapes(CqlBatchCatalog* c)
{
  if (!c) return 0;
  pthread_mutex_lock(&c->lock);
  uint32_t n = c->shapes;
  pthread_mutex_unlock(&c->lock);
  return n;
}

/* What a launch over the catalog compiles: its shapes, column types and summed columns, as they stood. */
typedef struct
{
  uint32_t shapes;
  char* exprs[CQL_BATCH_CATALOG_SHAPES];
  uint32_t sites[CQL_BATCH_CATALOG_SHAPES];
  uint32_t masks[CQL_BATCH_CATALOG_SHAPES];
  int types[CQL_BATCH_CATALOG_SHAPES * CQLOPS_MAX_BINDINGS];
  uint32_t sums[CQL_BATCH_CATALOG_SHAPES];
  int slot_type[CQLOPS_MAX_BINDINGS];
  uint32_t sum_mask;
  uint64_t version;
} CatalogView;

/* Maps the batch's shapes to catalog entries (adding the new ones) and takes a view of the catalog.
   0 when the catalog cannot take them (full, or a column read as another type): the batch then runs
   without it. Entries are never removed, so the view's strings stay valid while the catalog lives. */
static int catalog_map(CqlBatchCatalog* c, uint32_t shapes, char** exprs, const uint64_t* keys, const uint32_t* sites,
                       const uint32_t* masks, const int* types, const uint32_t* sums, const int* slot_type, uint32_t sum_mask,
                       uint32_t* out_index, CatalogView* view)
{
  int ok = 1;
  pthread_mutex_lock(&c->lock);
  for (int t = 0; t < CQLOPS_MAX_BINDINGS; t++)
    if (slot_type[t] && c->slot_type[t] && c->slot_type[t] != slot_type[t]) ok = 0;
  uint32_t added = 0;
  for (uint32_t s = 0; ok && s < shapes; s++)
  {
    uint32_t k = 0;
    while (k < c->shapes && !(c->keys[k] == keys[s] && !strcmp(c->exprs[k], exprs[s]))) k++;
    if (k == c->shapes)
    {
      if (k + added >= CQL_BATCH_CATALOG_SHAPES)
      {
        ok = 0;
        break;
      }
      k = c->shapes + added;
      added++;
    }
    out_index[s] = k;
  }
  if (ok)
  {
    /* the new shapes, in the order the batch met them */
    for (uint32_t s = 0; s < shapes; s++)
    {
      if (out_index[s] < c->shapes) continue;
      uint32_t k = out_index[s];
      size_t n = strlen(exprs[s]) + 1;
      char* e = (char*)malloc(n);
      if (!e)
      {
        ok = 0;
        break;
      }
      memcpy(e, exprs[s], n);
      c->keys[k] = keys[s];
      c->exprs[k] = e;
      c->sites[k] = sites[s];
      c->masks[k] = masks[s];
      memcpy(&c->types[k * CQLOPS_MAX_BINDINGS], &types[s * CQLOPS_MAX_BINDINGS], sizeof(int) * CQLOPS_MAX_BINDINGS);
      c->sums[k] = 0;
      c->shapes = k + 1;
      c->version++;
    }
    for (uint32_t s = 0; ok && s < shapes; s++)
    {
      uint32_t k = out_index[s];
      if ((c->sums[k] | sums[s]) != c->sums[k])
      {
        c->sums[k] |= sums[s];
        c->version++;
      }
    }
  }
  if (ok)
  {
    for (int t = 0; t < CQLOPS_MAX_BINDINGS; t++)
      if (slot_type[t] && !c->slot_type[t])
      {
        c->slot_type[t] = slot_type[t];
        c->version++;
      }
    if ((c->sum_mask | sum_mask) != c->sum_mask)
    {
      c->sum_mask |= sum_mask;
      c->version++;
    }
    view->shapes = c->shapes;
    memcpy(view->exprs, c->exprs, sizeof(c->exprs));
    memcpy(view->sites, c->sites, sizeof(c->sites));
    memcpy(view->masks, c->masks, sizeof(c->masks));
    memcpy(view->types, c->types, sizeof(c->types));
    memcpy(view->sums, c->sums, sizeof(c->sums));
    memcpy(view->slot_type, c->slot_type, sizeof(c->slot_type));
    view->sum_mask = c->sum_mask;
    view->version = c->version;
  }
  pthread_mutex_unlock(&c->lock);
  return ok;
}

/* ---- the operator ---- */

enum { BATCH_RUN = 0, BATCH_SOURCE = 1, BATCH_PREPARE = 2, BATCH_CUBE_BUILD_SOURCE = 3, BATCH_CUBE_ANSWER_SOURCE = 4, BATCH_PERSIST = 5 };

/* the persistent form's submission of one planned batch (defined with the persistent form below) */
typedef struct
{
  const CatalogView* view;
  uint32_t scan_n;
  const uint32_t* order;
  const uint32_t* shape_of;
  const Thr* thr;
  const double* qconst;
  const uint32_t* qsum_ordered;
  const uint32_t* qsum;
  const double* col_scale;
  const int64_t* col_shift;
  uint32_t need, sums;
  const int* sum_cols;
  uint32_t sum_col_count;
} PersistJob;
static __thread CqlBatchPersist* tl_persist;
static int persist_submit(CqlBatchPersist* P, const PersistJob* j, uint64_t* out_counts, double* out_sums, char* why, size_t why_cap);

/* The operator; with BATCH_SOURCE the source of its first launch, with BATCH_PREPARE its kernel compiled
   and the shapes entered in the catalog (neither does device work on the table). */
static int batch_run(CqlBatchCatalog* catalog, const CqlProgram* const* programs, uint32_t query_count, const CqlColumn* columns,
                     uint32_t column_count, const int32_t* sum_columns, uint32_t rows_per_thread, uint64_t* out_counts, double* out_sums,
                     uint32_t* out_shapes, int mode, char* src_out, uint64_t src_cap, uint64_t* src_len, int allow_cubes)
{
  cqlops_note_error("");
  if (query_count == 0) return 1;
  if (column_count == 0 || column_count > CQLOPS_MAX_BINDINGS) return refuse("1 to 10 columns");
  /* 0: the shared-memory tile form; 4, 8 or 16: the register form with that many rows per thread (the
     cube-source modes carry the table pass here instead) */
  uint32_t cube_pass = rows_per_thread;
  /* the form: rows per thread in the low byte, the register form's block size / 256 in the next (1 or 2) */
  uint32_t block = ((rows_per_thread >> 8) & 0xffu) == 2u ? 512u : 256u;
  int persistent_source = mode == BATCH_SOURCE && ((rows_per_thread >> 16) & 1u);   /* the persistent form's source */
  rows_per_thread &= 0xffu;
  if (rows_per_thread != 0 && rows_per_thread != 4 && rows_per_thread != 8 && rows_per_thread != 16) rows_per_thread = 8;
  uint64_t rows = columns[0].rows;
  if (!cqlops_rows_fit(rows)) return 0;
  for (uint32_t c = 0; c < column_count; c++)
  {
    const CqlColumn* col = &columns[c];
    if (col->rows != rows || (!col->buffer && mode == BATCH_RUN) || col->width != 0 || col->type == CQLOPS_TYPE_STRING8)
      return refuse("batched columns are full-width numeric columns of one length");
  }
  if (rows == 0 && (mode == BATCH_RUN || mode == BATCH_PERSIST))
  {
    /* an empty table: every query counts 0 rows and sums nothing (no device work) */
    for (uint32_t q = 0; q < query_count; q++)
    {
      out_counts[q] = 0;
      if (out_sums) out_sums[q] = 0.0;
    }
    if (out_shapes) *out_shapes = 0;
    return 1;
  }
  /* per query: rebound program, shape, thresholds, literals */
  CqlProgram* rb = (CqlProgram*)malloc(sizeof(CqlProgram));
  uint32_t* shape_of = (uint32_t*)malloc(query_count * 4);
  uint32_t* order = (uint32_t*)malloc(query_count * 4);
  Thr* thr = (Thr*)calloc((size_t)query_count * BATCH_MAX_SITES, sizeof(Thr));
  double* qconst = (double*)calloc((size_t)query_count * BATCH_MAX_CONSTS, sizeof(double));
  uint32_t* qsum = (uint32_t*)malloc(query_count * 4);
  char* exprs[BATCH_MAX_SHAPES];
  uint32_t shape_sites[BATCH_MAX_SHAPES];
  uint64_t shape_keys[BATCH_MAX_SHAPES];
  uint32_t shape_mask[BATCH_MAX_SHAPES];
  uint32_t shape_sums[BATCH_MAX_SHAPES];
  int* shape_types = (int*)calloc(BATCH_MAX_SHAPES * CQLOPS_MAX_BINDINGS, sizeof(int));
  CqlBatchSite* shape_site_list = (CqlBatchSite*)malloc((size_t)BATCH_MAX_SHAPES * BATCH_MAX_SITES * sizeof(CqlBatchSite));
  struct
  {
    uint32_t* w;
    uint32_t n;
  } shape_words[BATCH_MAX_SHAPES];
  uint32_t shapes = 0;
  int slot_type[CQLOPS_MAX_BINDINGS] = { 0 };
  int ok = rb && shape_of && order && thr && qconst && qsum && shape_types && shape_site_list;
  char why[160] = "";
  for (uint32_t q = 0; ok && q < query_count; q++)
  {
    const CqlProgram* p = programs[q];
    if (!p || p->const_count > BATCH_MAX_CONSTS || !rebind(p, column_count, rb))
    {
      snprintf(why, sizeof(why), "query %u cannot be batched (strings, or more than %d literals)", q, BATCH_MAX_CONSTS);
      ok = 0;
      break;
    }
    /* a shape is its rebound bytecode: a query whose words match a shape's takes its predicate, sites
       and column types without generating them again */
    uint64_t h = words_hash(rb);
    uint32_t s = 0;
    while (s < shapes && !(shape_keys[s] == h && shape_words[s].n == rb->word_count &&
                           !memcmp(shape_words[s].w, rb->words, rb->word_count * sizeof(uint32_t))))
      s++;
    if (s == shapes)
    {
      if (shapes == BATCH_MAX_SHAPES)
      {
        snprintf(why, sizeof(why), "more than %d query shapes in one batch", BATCH_MAX_SHAPES);
        ok = 0;
        break;
      }
      uint32_t site_count = 0;
      int st[CQLOPS_MAX_BINDINGS];
      char* expr = NULL;
      if (!cql_codegen_batch_predicate(rb, &shape_site_list[(uint64_t)s * BATCH_MAX_SITES], BATCH_MAX_SITES, &site_count, st, &expr, why,
                                       sizeof(why)))
      {
        ok = 0;
        break;
      }
      shape_words[s].w = (uint32_t*)malloc(rb->word_count * sizeof(uint32_t) + 4);
      if (!shape_words[s].w)
      {
        free(expr);
        ok = 0;
        break;
      }
      memcpy(shape_words[s].w, rb->words, rb->word_count * sizeof(uint32_t));
      shape_words[s].n = rb->word_count;
      shape_keys[s] = h;
      exprs[s] = expr;
      shape_sites[s] = site_count;
      shape_mask[s] = 0;
      shape_sums[s] = 0;
      for (int d = 0; d < CQLOPS_MAX_BINDINGS; d++)
      {
        shape_types[s * CQLOPS_MAX_BINDINGS + d] = st[d];
        if (st[d]) shape_mask[s] |= 1u << d;
      }
      for (int d = 0; d < CQLOPS_MAX_BINDINGS; d++)
      {
        if (!st[d]) continue;
        if (slot_type[d] && slot_type[d] != st[d])
        {
          snprintf(why, sizeof(why), "column %d read as two types", d);
          ok = 0;
        }
        slot_type[d] = st[d];
      }
      shapes++;
    }
    shape_of[q] = s;
    const CqlBatchSite* sites = &shape_site_list[(uint64_t)s * BATCH_MAX_SITES];
    uint32_t site_count = shape_sites[s];
    for (uint32_t i = 0; i < site_count; i++)
    {
      double c = const_value(p, sites[i].const_index);
      int t = (int)sites[i].col_type;
      Thr* th = &thr[(uint64_t)q * BATCH_MAX_SITES + i];
      if (t == CQLOPS_TYPE_F32) thr_f32(c, (int)sites[i].op, th);
      else if (t == CQLOPS_TYPE_F64) thr_f64(c, (int)sites[i].op, th);
      else thr_int(c, (int)sites[i].op, t == CQLOPS_TYPE_I32 || t == 9, th);
    }
    for (uint32_t i = 0; i < p->const_count; i++) qconst[(uint64_t)q * BATCH_MAX_CONSTS + i] = const_value(p, i);
    int32_t sc = sum_columns ? sum_columns[q] : -1;
    if (sc >= (int32_t)column_count)
    {
      snprintf(why, sizeof(why), "query %u sums a column outside the table", q);
      ok = 0;
      break;
    }
    qsum[q] = sc < 0 ? 0xffffffffu : (uint32_t)sc;
    if (sc >= 0) shape_sums[s] |= 1u << sc;
  }
  /* summed columns: loaded, scaled by 2^k with k from the column's range */
  uint32_t sm_count = cqlcuda_sm_count();
  double col_scale[CQLOPS_MAX_BINDINGS] = { 0 };
  int64_t col_shift[CQLOPS_MAX_BINDINGS] = { 0 };
  uint32_t sum_mask = 0;
  for (uint32_t q = 0; ok && q < query_count; q++)
  {
    if (qsum[q] == 0xffffffffu) continue;
    int c = (int)qsum[q];
    if ((sum_mask >> c) & 1u) continue;
    const CqlColumn* col = &columns[c];
    if (!col->has_range)
    {
      snprintf(why, sizeof(why), "a summed column needs its range");
      ok = 0;
      break;
    }
    if (!slot_type[c]) slot_type[c] = (int)col->type;
    double m = fabs(col->zone_min) > fabs(col->zone_max) ? fabs(col->zone_min) : fabs(col->zone_max);
    int e = 0;
    if (m > 0.0) frexp(m, &e);   /* m < 2^e */
    /* the rows one accumulator takes, the most any form takes: in the register form a warp's passes over
       the grid (32 lanes x rows per thread each), in the tile form a CTA's tiles (at most one SM's share
       of the rows and two tiles, whatever the CTAs per SM). One bound for every form gives every form the
       same scale, so a query's sum is the same integer whichever form (or the autotuner's choice) runs
       it - and the cube form, which adds the same summands to 128-bit cell totals. */
    uint64_t per_pass = (uint64_t)(sm_count ? sm_count : 152) * BATCH_CTAS_PER_SM * QE_GPU_WORKGROUP_SIZE;
    uint64_t warp_rows = rows / (sm_count ? sm_count : 152) + 2048;
    for (uint32_t rpt = 4; rpt <= 16; rpt *= 2)
    {
      uint64_t groups = (rows + rpt - 1) / rpt;
      uint64_t w = ((groups + per_pass - 1) / per_pass) * 32 * rpt;
      if (w > warp_rows) warp_rows = w;
    }
    int wr = 0;
    frexp((double)warp_rows, &wr);   /* warp_rows < 2^wr */
    col_scale[c] = ldexp(1.0, 62 - e - wr);
    col_shift[c] = 62 - e - wr;
    sum_mask |= 1u << c;
  }
  /* what the launches compile: this batch's shapes, or the catalog's */
  uint32_t launch_shapes = shapes;
  char** launch_exprs = exprs;
  uint32_t* launch_sites = shape_sites;
  uint32_t* launch_masks = shape_mask;
  int* launch_shape_types = shape_types;
  uint32_t* launch_shape_sums = shape_sums;
  int* launch_types = slot_type;
  uint32_t launch_sums = sum_mask;
  CatalogView* view = NULL;
  if (ok && catalog)
  {
    view = (CatalogView*)malloc(sizeof(CatalogView));
    uint32_t index[BATCH_MAX_SHAPES];
    if (view &&
        catalog_map(catalog, shapes, exprs, shape_keys, shape_sites, shape_mask, shape_types, shape_sums, slot_type, sum_mask, index, view))
    {
      for (uint32_t q = 0; q < query_count; q++) shape_of[q] = index[shape_of[q]];
      launch_shapes = view->shapes;
      launch_exprs = view->exprs;
      launch_sites = view->sites;
      launch_masks = view->masks;
      launch_shape_types = view->types;
      launch_shape_sums = view->sums;
      launch_types = view->slot_type;
      launch_sums = view->sum_mask;
    }
  }
  int sum_cols[CQLOPS_MAX_BINDINGS];
  uint32_t sum_col_count = 0;
  for (int c = 0; c < CQLOPS_MAX_BINDINGS; c++)
    if ((launch_sums >> c) & 1u) sum_cols[sum_col_count++] = c;
  /* the cube plan over the launch shapes, and the queries it answers */
  CubePlan* plan = NULL;
  int cube_of[BATCH_MAX_SHAPES];
  for (uint32_t sh = 0; sh < BATCH_MAX_SHAPES; sh++) cube_of[sh] = -1;
  int cube_source_mode = mode == BATCH_CUBE_BUILD_SOURCE || mode == BATCH_CUBE_ANSWER_SOURCE;
  if (ok && allow_cubes && (mode == BATCH_RUN || mode == BATCH_PREPARE || cube_source_mode))
  {
    plan = (CubePlan*)malloc(sizeof(CubePlan));
    if (plan) cube_plan(launch_shapes, launch_masks, launch_shape_types, launch_shape_sums, columns, column_count, plan, cube_of);
    if (plan && plan->cubes == 0)
    {
      free(plan);
      plan = NULL;
    }
  }
  /* a table pass costs about as much as a handful of queries on the scan (it reads the cubes' columns
     and adds every row to each table): fewer cube-answerable queries than CUBE_MIN_QUERIES stay on the scan */
  if (plan && mode == BATCH_RUN)
  {
    uint32_t answerable = 0;
    for (uint32_t q = 0; q < query_count; q++) answerable += cube_of[shape_of[q]] >= 0;
    if (answerable < CUBE_MIN_QUERIES)
    {
      free(plan);
      plan = NULL;
    }
  }
  uint32_t* cube_q = (uint32_t*)malloc(query_count * 4);
  ok = ok && cube_q;
  uint32_t cube_n = 0;
  uint32_t need = 0, scan_sums = 0, cube_sums = 0, cube_need = 0, cube_load = 0;
  for (uint32_t q = 0; ok && q < query_count; q++)
  {
    uint32_t bit = qsum[q] == 0xffffffffu ? 0u : 1u << qsum[q];
    if (plan && cube_of[shape_of[q]] >= 0)
    {
      cube_q[cube_n++] = q;
      cube_sums |= bit;
      cube_need |= 1u << cube_of[shape_of[q]];
      cube_load |= plan->cube[cube_of[shape_of[q]]].mask | bit;
    }
    else
    {
      need |= launch_masks[shape_of[q]] | bit;
      scan_sums |= bit;
    }
  }
  uint32_t scan_n = query_count - cube_n;
  /* the scan's queries grouped by (launch) shape */
  uint32_t* shape_count = (uint32_t*)calloc(launch_shapes + 1, 4);
  ok = ok && shape_count;
  if (ok)
  {
    for (uint32_t q = 0; q < query_count; q++)
      if (!(plan && cube_of[shape_of[q]] >= 0)) shape_count[shape_of[q]]++;
    uint32_t* start = (uint32_t*)malloc((launch_shapes + 1) * 4);
    if (!start) ok = 0;
    else
    {
      uint32_t run = 0;
      for (uint32_t sh = 0; sh < launch_shapes; sh++)
      {
        start[sh] = run;
        run += shape_count[sh];
      }
      for (uint32_t q = 0; q < query_count; q++)
        if (!(plan && cube_of[shape_of[q]] >= 0)) order[start[shape_of[q]]++] = q;
      free(start);
    }
  }
  /* thresholds, literals and sums of the scan's queries in shape order */
  uint32_t nalloc = scan_n ? scan_n : 1;
  Thr* thr_o = ok ? (Thr*)malloc((size_t)nalloc * BATCH_MAX_SITES * sizeof(Thr)) : NULL;
  double* qc_o = ok ? (double*)malloc((size_t)nalloc * BATCH_MAX_CONSTS * sizeof(double)) : NULL;
  uint32_t* qs_o = ok ? (uint32_t*)malloc(nalloc * 4) : NULL;
  ok = ok && thr_o && qc_o && qs_o;
  if (ok)
    for (uint32_t i = 0; i < scan_n; i++)
    {
      uint32_t q = order[i];
      memcpy(&thr_o[(uint64_t)i * BATCH_MAX_SITES], &thr[(uint64_t)q * BATCH_MAX_SITES], sizeof(Thr) * BATCH_MAX_SITES);
      memcpy(&qc_o[(uint64_t)i * BATCH_MAX_CONSTS], &qconst[(uint64_t)q * BATCH_MAX_CONSTS], sizeof(double) * BATCH_MAX_CONSTS);
      qs_o[i] = qsum[q];
    }
  uint64_t* folded = ok && mode == BATCH_RUN ? (uint64_t*)malloc((size_t)nalloc * 24) : NULL;
  ok = ok && (folded || mode != BATCH_RUN);
  /* one launch per slice of at most CQL_BATCH_LAUNCH_QUERIES queries: its shapes (all of the catalog's,
     with a catalog) and where each starts */
  uint32_t begin[BATCH_MAX_SHAPES + 1];
  char* slice_exprs[BATCH_MAX_SHAPES];
  uint32_t slice_sites[BATCH_MAX_SHAPES];
#define SLICE_SHAPES(first, nq, ns)                                                   \
  do                                                                                  \
  {                                                                                   \
    ns = 0;                                                                           \
    if (view && launch_exprs == view->exprs)                                          \
    {                                                                                 \
      uint32_t at_ = 0;                                                               \
      for (uint32_t s_ = 0; s_ < launch_shapes; s_++)                                 \
      {                                                                               \
        while (at_ < (nq) && shape_of[order[(first) + at_]] < s_) at_++;              \
        begin[s_] = at_;                                                              \
        slice_exprs[s_] = launch_exprs[s_];                                           \
        slice_sites[s_] = launch_sites[s_];                                           \
      }                                                                               \
      ns = launch_shapes;                                                             \
    }                                                                                 \
    else                                                                              \
      for (uint32_t i_ = 0; i_ < (nq); i_++)                                          \
      {                                                                               \
        uint32_t s_ = shape_of[order[(first) + i_]];                                  \
        if (ns == 0 || slice_exprs[ns - 1] != launch_exprs[s_])                       \
        {                                                                             \
          slice_exprs[ns] = launch_exprs[s_];                                         \
          slice_sites[ns] = launch_sites[s_];                                         \
          begin[ns] = i_;                                                             \
          ns++;                                                                       \
        }                                                                             \
      }                                                                               \
    begin[ns] = (nq);                                                                 \
  } while (0)
  /* the cube kernels (compiled or found in the cache) */
  CqlKernel* cube_build[CUBE_MAX] = { NULL };
  CqlKernel* cube_answer = NULL;
  if (cube_source_mode)
  {
    /* the cube kernels' sources, for a compile check (no device work) */
    char* src = NULL;
    if (ok && plan && mode == BATCH_CUBE_ANSWER_SOURCE) src = cube_answer_source(plan, launch_exprs, launch_sites, launch_shapes, cube_of);
    else if (ok && plan && cube_pass < plan->passes) src = cube_build_source(plan, cube_pass, launch_types);
    else if (ok && plan) refuse("no such table pass");
    if (src)
    {
      uint64_t n = strlen(src);
      if (src_len) *src_len = n;
      if (src_out && src_cap) snprintf(src_out, src_cap, "%s", src);
      ok = !(src_out && n + 1 > src_cap);
    }
    else
    {
      if (ok && !plan) refuse("no query of the batch can be answered from a cube");
      ok = 0;
    }
    free(src);
    if (out_shapes) *out_shapes = cube_n;
    mode = BATCH_SOURCE + 100;   /* nothing below runs */
    free(plan);
    plan = NULL;
  }
  if (ok && plan)
  {
    char name[64];
    for (uint32_t p = 0; ok && p < plan->passes; p++)
    {
      char* src = cube_build_source(plan, p, launch_types);
      if (src)
      {
        snprintf(name, sizeof(name), "qk_cube_%016llx", (unsigned long long)fnv_str(src));
        cube_build[p] = cqlcuda_kernel_alloc(name, strlen(name));
        if (!cube_build[p]) cube_build[p] = cqlcuda_kernel_alloc_from_image(name, strlen(name), src, strlen(src));
      }
      free(src);
      if (!cube_build[p]) ok = 0;
    }
    char* asrc = ok ? cube_answer_source(plan, launch_exprs, launch_sites, launch_shapes, cube_of) : NULL;
    if (asrc)
    {
      snprintf(name, sizeof(name), "qk_cubea_%016llx", (unsigned long long)fnv_str(asrc));
      cube_answer = cqlcuda_kernel_alloc(name, strlen(name));
      if (!cube_answer) cube_answer = cqlcuda_kernel_alloc_from_image(name, strlen(name), asrc, strlen(asrc));
    }
    free(asrc);
    if (!cube_answer) ok = 0;
  }
  if (ok && (mode == BATCH_SOURCE || mode == BATCH_PREPARE) && (scan_n || view))
  {
    uint32_t nq = scan_n < CQL_BATCH_LAUNCH_QUERIES ? scan_n : CQL_BATCH_LAUNCH_QUERIES;
    uint32_t ns;
    SLICE_SHAPES(0, nq, ns);
    char* src = launch_source(slice_exprs, slice_sites, ns, launch_types, sum_cols, sum_col_count, rows_per_thread, block, persistent_source);
    ok = src != NULL;
    if (ok && mode == BATCH_SOURCE)
    {
      uint64_t n = strlen(src);
      if (src_len) *src_len = n;
      if (src_out && src_cap) snprintf(src_out, src_cap, "%s", src);
      if (src_out && n + 1 > src_cap) ok = 0;
    }
    else if (ok)
    {
      char name[64];
      snprintf(name, sizeof(name), "qk_batch_%016llx", (unsigned long long)fnv_str(src));
      size_t nlen = strlen(name);
      ok = cqlcuda_kernel_alloc(name, nlen) || cqlcuda_kernel_alloc_from_image(name, nlen, src, strlen(src));
    }
    free(src);
  }
  if (ok && (mode == BATCH_SOURCE || mode == BATCH_PREPARE) && out_shapes) *out_shapes = shapes;
  if (mode == BATCH_PERSIST)
  {
    /* the persistent form: the batch's parameters into a ring slot of the kernel compiled for the catalog */
    if (ok && (!view || launch_exprs != view->exprs || scan_n != query_count || scan_n > CQL_BATCH_LAUNCH_QUERIES))
    {
      snprintf(why, sizeof(why), "the persistent scan takes at most %d queries of catalog shapes", CQL_BATCH_LAUNCH_QUERIES);
      ok = 0;
    }
    if (ok)
    {
      PersistJob job = { view, scan_n, order, shape_of, thr_o, qc_o, qs_o, qsum, col_scale, col_shift, need, scan_sums, sum_cols, sum_col_count };
      ok = persist_submit(tl_persist, &job, out_counts, out_sums, why, sizeof(why));
      if (ok && out_shapes) *out_shapes = shapes;
    }
  }
  int launch = ok && mode == BATCH_RUN;
  /* one upload of every launch parameter: the scales (doubles at 0..), then their exponents (64-bit
     integers at 16..), the scan's thresholds, literals and summed columns in shape order, each slice's shape
     starts, then the cube queries' thresholds, literals and (shape, cube, summed column); each part on a
     16-byte boundary */
  uint32_t slices = (scan_n + CQL_BATCH_LAUNCH_QUERIES - 1) / CQL_BATCH_LAUNCH_QUERIES;
  const uint64_t off_thr = 256;
  const uint64_t off_qc = off_thr + (uint64_t)scan_n * BATCH_MAX_SITES * sizeof(Thr);
  const uint64_t off_qs = off_qc + (uint64_t)scan_n * BATCH_MAX_CONSTS * 8;
  const uint64_t off_begin = off_qs + (((uint64_t)scan_n * 4 + 15) & ~15ull);
  const uint64_t begin_stride = ((BATCH_MAX_SHAPES + 1) * 4 + 15) & ~15ull;
  const uint64_t off_cthr = off_begin + (uint64_t)slices * begin_stride;
  const uint64_t off_cqc = off_cthr + (uint64_t)cube_n * BATCH_MAX_SITES * sizeof(Thr);
  const uint64_t off_cmeta = off_cqc + (uint64_t)cube_n * BATCH_MAX_CONSTS * 8;
  const uint64_t param_bytes = off_cmeta + (((uint64_t)cube_n * 4 + 15) & ~15ull) + 16;
  unsigned char* params = launch ? (unsigned char*)calloc(1, param_bytes) : NULL;
  if (launch && !params) ok = 0;
  if (params)
  {
    memcpy(params, col_scale, sizeof(col_scale));
    memcpy(params + 128, col_shift, sizeof(col_shift));
    memcpy(params + off_thr, thr_o, (size_t)scan_n * BATCH_MAX_SITES * sizeof(Thr));
    memcpy(params + off_qc, qc_o, (size_t)scan_n * BATCH_MAX_CONSTS * 8);
    memcpy(params + off_qs, qs_o, (size_t)scan_n * 4);
    for (uint32_t i = 0; i < cube_n; i++)
    {
      uint32_t q = cube_q[i];
      const Cube* cu = &plan->cube[cube_of[shape_of[q]]];
      uint32_t j = 0;
      while (j < cu->nsum && (uint32_t)cu->sum_slot[j] != qsum[q]) j++;
      uint32_t meta = shape_of[q] | ((uint32_t)cube_of[shape_of[q]] << 8) | ((qsum[q] == 0xffffffffu || j == cu->nsum) ? 0u : (j + 1u) << 16);
      memcpy(params + off_cthr + (uint64_t)i * BATCH_MAX_SITES * sizeof(Thr), &thr[(uint64_t)q * BATCH_MAX_SITES], BATCH_MAX_SITES * sizeof(Thr));
      memcpy(params + off_cqc + (uint64_t)i * BATCH_MAX_CONSTS * 8, &qconst[(uint64_t)q * BATCH_MAX_CONSTS], BATCH_MAX_CONSTS * 8);
      memcpy(params + off_cmeta + (uint64_t)i * 4, &meta, 4);
    }
  }
  uint32_t per_sm = rows_per_thread ? register_ctas_per_sm(block) : tiled_layout(launch_types, sum_col_count).per_sm;
  uint64_t ctas = (uint64_t)(sm_count ? sm_count : 152) * per_sm;
  uint32_t widest = scan_n < CQL_BATCH_LAUNCH_QUERIES ? scan_n : CQL_BATCH_LAUNCH_QUERIES;
  const uint64_t cube_out_bytes = 16 + (uint64_t)cube_n * 24;   /* the error word, then (count, lo, hi) per cube query */
  uint64_t* cube_out = launch && cube_n ? (uint64_t*)malloc(cube_out_bytes) : NULL;
  if (launch && cube_n && !cube_out) ok = 0;
  CqlBuffer* param_buf = launch && ok ? pooled("batch_params", param_bytes, CQLCUDA_BUFFER_WRITE) : NULL;
  CqlBuffer* out_buf = launch && ok && scan_n ? pooled("batch_folded", (uint64_t)scan_n * 24, CQLCUDA_BUFFER_READ_WRITE) : NULL;
  CqlBuffer* parts = launch && ok && scan_n ? pooled("batch_partials", ctas * widest * 24, CQLCUDA_BUFFER_READ_WRITE) : NULL;
  CqlBuffer* tables = launch && ok && cube_n ? pooled("batch_cube_tables", plan->words * 8, CQLCUDA_BUFFER_READ_WRITE) : NULL;
  CqlBuffer* cube_out_buf = launch && ok && cube_n ? pooled("batch_cube_out", cube_out_bytes, CQLCUDA_BUFFER_READ_WRITE) : NULL;
  CqlKernel* fold = launch && scan_n ? cqlcuda_kernel_alloc("cql_batch_fold", 14) : NULL;
  if (launch)
    ok = ok && param_buf && (!scan_n || (out_buf && parts && fold)) && (!cube_n || (tables && cube_out_buf && cube_answer));
  launch = launch && ok;
  /* each slice's kernel, compiled (or found) before anything is queued; with a catalog one for all */
  CqlKernel** kernels = launch ? (CqlKernel**)calloc(slices ? slices : 1, sizeof(CqlKernel*)) : NULL;
  uint32_t* slice_ns = launch ? (uint32_t*)calloc(slices ? slices : 1, 4) : NULL;
  if (launch && (!kernels || !slice_ns)) ok = 0;
  CqlKernel* shared_k = NULL;
  for (uint32_t sl = 0; launch && ok && sl < slices; sl++)
  {
    uint32_t first = sl * CQL_BATCH_LAUNCH_QUERIES;
    uint32_t nq = scan_n - first < CQL_BATCH_LAUNCH_QUERIES ? scan_n - first : CQL_BATCH_LAUNCH_QUERIES;
    uint32_t ns;
    SLICE_SHAPES(first, nq, ns);
    memcpy(params + off_begin + sl * begin_stride, begin, (ns + 1) * 4);
    slice_ns[sl] = ns;
    CqlKernel* k = shared_k;
    if (!k)
    {
      char* src = launch_source(slice_exprs, slice_sites, ns, launch_types, sum_cols, sum_col_count, rows_per_thread, block, 0);
      if (!src)
      {
        ok = 0;
        break;
      }
      char name[64];
      snprintf(name, sizeof(name), "qk_batch_%016llx", (unsigned long long)fnv_str(src));
      size_t nlen = strlen(name);
      k = cqlcuda_kernel_alloc(name, nlen);
      if (!k) k = cqlcuda_kernel_alloc_from_image(name, nlen, src, strlen(src));
      free(src);
      if (!k)
      {
        ok = 0;
        break;
      }
      if (view && launch_exprs == view->exprs) shared_k = k;
    }
    kernels[sl] = k;
  }
#undef SLICE_SHAPES
  /* one batch: the upload, the cube pass and answers, every slice's scan and fold, the read-backs; one wait.
     It runs as the CUDA graph of its plan shape: a batch of the same shapes, query count and buffers
     replays the graph captured for it, with this batch's thresholds as the uploaded bytes. */
  if (launch && ok)
  {
    CqlBatch* b = cqlcuda_batch_begin_graph(param_bytes, (uint64_t)scan_n * 24 + (cube_n ? cube_out_bytes : 0), 0x62617463685f7363ull);
    cqlcuda_batch_buffer_write(b, param_buf, params, param_bytes);
    if (cube_n)
    {
      cqlcuda_batch_buffer_zero(b, tables, plan->words * 8);
      cqlcuda_batch_buffer_zero(b, cube_out_buf, 16);
      for (uint32_t p = 0; p < plan->passes; p++)
      {
        int wanted = 0;
        for (uint32_t c = 0; c < plan->cubes; c++) wanted |= plan->cube[c].pass == p && ((cube_need >> c) & 1u);
        if (!wanted) continue;   /* no query of the batch reads this pass's cubes */
        CqlKernel* kb = cube_build[p];
        cqlcuda_kernel_set_arg_buffer_range(kb, 0, param_buf, 0, 256);
        cqlcuda_kernel_set_arg_buffer(kb, 1, tables);
        cqlcuda_kernel_set_arg_buffer_range(kb, 2, cube_out_buf, 0, 16);
        for (uint32_t c = 0; c < CQLOPS_MAX_BINDINGS; c++)
          cqlcuda_kernel_set_arg_buffer(kb, 6 + c, columns[c < column_count ? c : 0].buffer);
        cqlcuda_kernel_set_arg_u64(kb, 0, rows);
        cqlcuda_kernel_set_arg_u64(kb, 1, cube_sums);
        cqlcuda_kernel_set_arg_u64(kb, 2, cube_need);
        cqlcuda_kernel_set_arg_u64(kb, 3, cube_load);
        cqlcuda_batch_kernel_execute(b, kb, (uint32_t)((sm_count ? sm_count : 152) * CUBE_THREADS), CUBE_THREADS);
      }
      cqlcuda_kernel_set_arg_buffer(cube_answer, 1, tables);
      cqlcuda_kernel_set_arg_buffer_range(cube_answer, 3, param_buf, off_cthr, off_cqc - off_cthr);
      cqlcuda_kernel_set_arg_buffer_range(cube_answer, 4, param_buf, off_cqc, off_cmeta - off_cqc);
      cqlcuda_kernel_set_arg_buffer_range(cube_answer, 5, param_buf, off_cmeta, (uint64_t)cube_n * 4);
      cqlcuda_kernel_set_arg_buffer_range(cube_answer, 6, cube_out_buf, 16, (uint64_t)cube_n * 24);
      cqlcuda_kernel_set_arg_u64(cube_answer, 0, cube_n);
      cqlcuda_batch_kernel_execute(b, cube_answer, cube_n * 256u, 256u);
    }
    for (uint32_t sl = 0; sl < slices; sl++)
    {
      uint32_t first = sl * CQL_BATCH_LAUNCH_QUERIES;
      uint32_t nq = scan_n - first < CQL_BATCH_LAUNCH_QUERIES ? scan_n - first : CQL_BATCH_LAUNCH_QUERIES;
      CqlKernel* k = kernels[sl];
      cqlcuda_kernel_set_arg_buffer_range(k, 0, param_buf, 0, 256);
      cqlcuda_kernel_set_arg_buffer_range(k, 1, param_buf, off_thr, off_qc - off_thr);
      cqlcuda_kernel_set_arg_buffer_range(k, 2, param_buf, off_qc, off_qs - off_qc);
      cqlcuda_kernel_set_arg_buffer_range(k, 3, param_buf, off_qs, (uint64_t)scan_n * 4);
      cqlcuda_kernel_set_arg_buffer_range(k, 4, param_buf, off_begin + sl * begin_stride, (slice_ns[sl] + 1) * 4);
      cqlcuda_kernel_set_arg_buffer_range(k, 5, parts, 0, ctas * nq * 24);
      for (uint32_t c = 0; c < CQLOPS_MAX_BINDINGS; c++)
        cqlcuda_kernel_set_arg_buffer(k, 6 + c, columns[c < column_count ? c : 0].buffer);
      cqlcuda_kernel_set_arg_u64(k, 0, rows);
      cqlcuda_kernel_set_arg_u64(k, 1, nq);
      cqlcuda_kernel_set_arg_u64(k, 2, first);
      cqlcuda_kernel_set_arg_u64(k, 3, (uint64_t)need | (uint64_t)scan_sums << 32);
      cqlcuda_kernel_set_arg_buffer_range(fold, 0, parts, 0, ctas * nq * 24);
      cqlcuda_kernel_set_arg_buffer_range(fold, 1, out_buf, (uint64_t)first * 24, (uint64_t)nq * 24);
      cqlcuda_kernel_set_arg_u64(fold, 0, nq);
      cqlcuda_kernel_set_arg_u64(fold, 1, ctas);
      cqlcuda_batch_buffer_zero(b, parts, ctas * nq * 24);
      cqlcuda_batch_kernel_execute(b, k, (uint32_t)(ctas * QE_GPU_WORKGROUP_SIZE), QE_GPU_WORKGROUP_SIZE);
      cqlcuda_batch_kernel_execute(b, fold, nq, QE_GPU_WORKGROUP_SIZE);
    }
    if (scan_n) cqlcuda_batch_buffer_read(b, out_buf, folded, (uint64_t)scan_n * 24);
    if (cube_n) cqlcuda_batch_buffer_read(b, cube_out_buf, cube_out, cube_out_bytes);
    ok = cqlcuda_batch_end(b);
  }
  free(params);
  free(kernels);
  free(slice_ns);
  if (launch && ok)
  {
    for (uint32_t i = 0; i < scan_n + cube_n; i++)
    {
      uint32_t q;
      uint64_t cnt, lo;
      int64_t hi;
      if (i < scan_n)
      {
        q = order[i];
        cnt = folded[i * 3];
        lo = folded[i * 3 + 1];
        hi = (int64_t)folded[i * 3 + 2];
      }
      else
      {
        uint32_t ci = i - scan_n;
        q = cube_q[ci];
        cnt = cube_out[2 + ci * 3];
        lo = cube_out[2 + ci * 3 + 1];
        hi = (int64_t)cube_out[2 + ci * 3 + 2];
      }
      out_counts[q] = cnt;
      if (!out_sums) continue;
      if (qsum[q] == 0xffffffffu)
      {
        out_sums[q] = 0.0;
        continue;
      }
      /* the 128-bit scaled sum, back to a double: hi * 2^64 + lo, then / 2^k */
      double v = (double)hi * 18446744073709551616.0 + (double)lo;
      out_sums[q] = v / col_scale[qsum[q]];
    }
    if (out_shapes) *out_shapes = shapes;
    /* a value outside its column's stated range left the cube pass: those queries run on the scan */
    if (cube_n && (uint32_t)cube_out[0] != 0u)
    {
      const CqlProgram** sub = (const CqlProgram**)malloc(cube_n * sizeof(*sub));
      int32_t* sub_sums = (int32_t*)malloc(cube_n * 4);
      uint64_t* sub_counts = (uint64_t*)malloc(cube_n * 8);
      double* sub_out = (double*)malloc(cube_n * 8);
      ok = sub && sub_sums && sub_counts && sub_out;
      for (uint32_t i = 0; ok && i < cube_n; i++)
      {
        sub[i] = programs[cube_q[i]];
        sub_sums[i] = qsum[cube_q[i]] == 0xffffffffu ? -1 : (int32_t)qsum[cube_q[i]];
      }
      if (ok)
        ok = batch_run(catalog, sub, cube_n, columns, column_count, sub_sums, rows_per_thread, sub_counts, sub_out, NULL, BATCH_RUN, NULL, 0,
                       NULL, 0);
      for (uint32_t i = 0; ok && i < cube_n; i++)
      {
        out_counts[cube_q[i]] = sub_counts[i];
        if (out_sums) out_sums[cube_q[i]] = sub_out[i];
      }
      free(sub);
      free(sub_sums);
      free(sub_counts);
      free(sub_out);
    }
  }
  else if (!ok && why[0])
    refuse(why);
  for (uint32_t sh = 0; sh < shapes; sh++)
  {
    free(exprs[sh]);
    free(shape_words[sh].w);
  }
  free(shape_site_list);
  free(view);
  free(plan);
  free(cube_q);
  free(cube_out);
  free(shape_types);
  free(rb);
  free(shape_of);
  free(order);
  free(thr);
  free(qconst);
  free(qsum);
  free(shape_count);
  free(thr_o);
  free(qc_o);
  free(qs_o);
  free(folded);
  return ok;
}

/* ---- the persistent form ---- */

#define PERSIST_SLOTS 4
#define PERSIST_WAIT_MS 5000

struct CqlBatchPersist
{
  pthread_mutex_t lock;
  CqlBatchCatalog* catalog;
  CqlColumn columns[CQLOPS_MAX_BINDINGS];
  uint32_t column_count;
  uint32_t rows_per_thread;
  uint32_t idle_us;
  uint64_t version;             /* the catalog version the kernel was compiled from */
  int compiled;
  CqlKernel* kernel;
  CqlPersistent* run;
  CqlBuffer* ring;              /* PERSIST_SLOTS sequence words */
  CqlBuffer* params;            /* PERSIST_SLOTS parameter slots */
  CqlBuffer* state;             /* tickets (64 bytes), then the accumulators */
  CqlBuffer* answers_buf;       /* page-locked host: the answers, then the done words */
  uint64_t* answers;
  uint64_t* done;
  uint64_t slot_bytes;
  unsigned char* staging;       /* each slot's parameters as copied (kept until the batch is done) */
  uint64_t seq_word[PERSIST_SLOTS + 1];
  uint64_t next_seq;
  uint64_t batches, launches, compiles;
  int broken;
};

/* a slot's layout: the scales and shifts (256 B), the header (nq, need | sums << 32) at 256, thresholds at
   512, literals, summed columns, shape starts (the generated entry computes the same offsets from NQ) */
static uint64_t persist_off_qc(void) { return 512ull + (uint64_t)CQL_BATCH_LAUNCH_QUERIES * BATCH_MAX_SITES * sizeof(Thr); }
static uint64_t persist_off_qs(void) { return persist_off_qc() + (uint64_t)CQL_BATCH_LAUNCH_QUERIES * BATCH_MAX_CONSTS * 8ull; }
static uint64_t persist_off_begin(void) { return persist_off_qs() + (((uint64_t)CQL_BATCH_LAUNCH_QUERIES * 4ull + 15ull) & ~15ull); }

static uint64_t persist_state_bytes(void) { return 64ull + (uint64_t)PERSIST_SLOTS * CQL_BATCH_LAUNCH_QUERIES * 24ull; }

CqlBatchPersist* cqlops_batch_persist_create(CqlBatchCatalog* catalog, const CqlColumn* columns, uint32_t column_count,
                                             uint32_t rows_per_thread, uint32_t idle_us)
{
  cqlops_note_error("");
  if (!catalog || !columns || column_count == 0 || column_count > CQLOPS_MAX_BINDINGS)
  {
    refuse("the persistent scan needs a catalog and 1 to 10 columns");
    return NULL;
  }
  if (rows_per_thread != 4 && rows_per_thread != 8 && rows_per_thread != 16)
  {
    refuse("the persistent scan takes 4, 8 or 16 rows per thread");
    return NULL;
  }
  if (!cqlops_rows_fit(columns[0].rows)) return NULL;
  for (uint32_t c = 0; c < column_count; c++)
    if (!columns[c].buffer || columns[c].rows != columns[0].rows || columns[c].width != 0)
    {
      refuse("batched columns are full-width numeric columns of one length");
      return NULL;
    }
  CqlBatchPersist* p = (CqlBatchPersist*)calloc(1, sizeof(CqlBatchPersist));
  if (!p) return NULL;
  pthread_mutex_init(&p->lock, NULL);
  p->catalog = catalog;
  memcpy(p->columns, columns, column_count * sizeof(CqlColumn));
  p->column_count = column_count;
  p->rows_per_thread = rows_per_thread;
  p->idle_us = idle_us ? idle_us : 2000;
  p->slot_bytes = (persist_off_begin() + (BATCH_MAX_SHAPES + 1) * 4 + 255) & ~255ull;
  p->ring = cqlcuda_buffer_alloc(PERSIST_SLOTS * 8, CQLCUDA_BUFFER_READ_WRITE, NULL);
  p->params = cqlcuda_buffer_alloc(PERSIST_SLOTS * p->slot_bytes, CQLCUDA_BUFFER_READ_WRITE, NULL);
  p->state = cqlcuda_buffer_alloc(persist_state_bytes(), CQLCUDA_BUFFER_READ_WRITE, NULL);
  void* host = NULL;
  p->answers_buf = cqlcuda_buffer_alloc_host_mapped((uint64_t)PERSIST_SLOTS * CQL_BATCH_LAUNCH_QUERIES * 24 + PERSIST_SLOTS * 8, &host);
  p->staging = (unsigned char*)calloc(PERSIST_SLOTS, p->slot_bytes);
  if (!p->ring || !p->params || !p->state || !p->answers_buf || !p->staging)
  {
    cqlops_batch_persist_destroy(p);
    return NULL;
  }
  p->answers = (uint64_t*)host;
  p->done = p->answers + (uint64_t)PERSIST_SLOTS * CQL_BATCH_LAUNCH_QUERIES * 3;
  /* the ring starts at 0 (no sequence number is 0) */
  uint64_t zero[PERSIST_SLOTS] = { 0 };
  cqlcuda_buffer_write(p->ring, zero, sizeof(zero));
  p->next_seq = 1;
  return p;
}

/* tells a running kernel to return (the stop word in the slot it waits on) and waits for it */
static int persist_stop(CqlBatchPersist* P)
{
  if (!P->run) return 1;
  if (cqlcuda_persistent_running(P->run) == 1)
  {
    P->seq_word[PERSIST_SLOTS] = ~0ull;
    cqlcuda_persistent_copy(P->run, P->ring, (P->next_seq % PERSIST_SLOTS) * 8, &P->seq_word[PERSIST_SLOTS], 8);
  }
  if (!cqlcuda_persistent_destroy(P->run, PERSIST_WAIT_MS)) return 0;
  P->run = NULL;
  /* the stop word must not stay where the next kernel looks */
  uint64_t ring[PERSIST_SLOTS] = { 0 };
  cqlcuda_buffer_write(P->ring, ring, sizeof(ring));
  return 1;
}

/* the kernel for the catalog as the job's view holds it */
static int persist_compile(CqlBatchPersist* P, const PersistJob* j)
{
  if (!persist_stop(P)) return refuse("the persistent scan did not return");
  char* src = batch_source((char**)j->view->exprs, j->view->sites, j->view->shapes, j->view->slot_type, j->sum_cols, j->sum_col_count,
                           P->rows_per_thread, 256, 1);
  if (!src) return 0;
  char name[64];
  snprintf(name, sizeof(name), "qk_persist_%016llx", (unsigned long long)fnv_str(src));
  size_t nlen = strlen(name);
  CqlKernel* k = cqlcuda_kernel_alloc(name, nlen);
  if (!k) k = cqlcuda_kernel_alloc_from_image(name, nlen, src, strlen(src));
  free(src);
  if (!k) return 0;
  P->run = cqlcuda_persistent_create(k, "cql_persist");
  if (!P->run) return 0;
  P->kernel = k;
  P->version = j->view->version;
  P->compiled = 1;
  P->compiles++;
  return 1;
}

/* launches the kernel (again), starting at sequence number `first`, with the accumulators and tickets clear */
static int persist_launch(CqlBatchPersist* P, uint64_t first)
{
  CqlKernel* k = P->kernel;
  cqlcuda_kernel_set_arg_buffer(k, 0, P->ring);
  cqlcuda_kernel_set_arg_buffer(k, 1, P->params);
  cqlcuda_kernel_set_arg_buffer_range(k, 2, P->state, 64, persist_state_bytes() - 64);
  cqlcuda_kernel_set_arg_buffer_range(k, 3, P->state, 0, 64);
  cqlcuda_kernel_set_arg_buffer_range(k, 4, P->answers_buf, 0, (uint64_t)PERSIST_SLOTS * CQL_BATCH_LAUNCH_QUERIES * 24);
  cqlcuda_kernel_set_arg_buffer_range(k, 5, P->answers_buf, (uint64_t)PERSIST_SLOTS * CQL_BATCH_LAUNCH_QUERIES * 24, PERSIST_SLOTS * 8);
  for (uint32_t c = 0; c < CQLOPS_MAX_BINDINGS; c++)
    cqlcuda_kernel_set_arg_buffer(k, 6 + c, P->columns[c < P->column_count ? c : 0].buffer);
  cqlcuda_kernel_set_arg_u64(k, 0, P->columns[0].rows);
  cqlcuda_kernel_set_arg_u64(k, 1, PERSIST_SLOTS);
  cqlcuda_kernel_set_arg_u64(k, 2, CQL_BATCH_LAUNCH_QUERIES);
  cqlcuda_kernel_set_arg_u64(k, 3, P->slot_bytes);
  cqlcuda_kernel_set_arg_u64(k, 4, P->idle_us);
  cqlcuda_kernel_set_arg_u64(k, 5, first);
  if (!cqlcuda_persistent_launch(P->run, 0, P->state, persist_state_bytes())) return 0;
  P->launches++;
  return 1;
}

static int persist_submit(CqlBatchPersist* P, const PersistJob* j, uint64_t* out_counts, double* out_sums, char* why, size_t why_cap)
{
  if (!P || P->broken)
  {
    snprintf(why, why_cap, "the persistent scan is not usable");
    return 0;
  }
  if (!P->compiled || P->version != j->view->version)
    if (!persist_compile(P, j)) return 0;
  uint64_t seq = P->next_seq;
  uint32_t slot = (uint32_t)(seq % PERSIST_SLOTS);
  /* the slot's parameters */
  unsigned char* sp = P->staging + (uint64_t)slot * P->slot_bytes;
  memcpy(sp, j->col_scale, CQLOPS_MAX_BINDINGS * sizeof(double));
  memset(sp + CQLOPS_MAX_BINDINGS * sizeof(double), 0, 128 - CQLOPS_MAX_BINDINGS * sizeof(double));
  memcpy(sp + 128, j->col_shift, CQLOPS_MAX_BINDINGS * sizeof(int64_t));
  uint64_t hdr[2] = { j->scan_n, (uint64_t)j->need | (uint64_t)j->sums << 32 };
  memcpy(sp + 256, hdr, sizeof(hdr));
  memcpy(sp + 512, j->thr, (size_t)j->scan_n * BATCH_MAX_SITES * sizeof(Thr));
  memcpy(sp + persist_off_qc(), j->qconst, (size_t)j->scan_n * BATCH_MAX_CONSTS * 8);
  memcpy(sp + persist_off_qs(), j->qsum_ordered, (size_t)j->scan_n * 4);
  /* where each catalog shape's queries start in the ordered list */
  uint32_t* begin = (uint32_t*)(sp + persist_off_begin());
  uint32_t at = 0;
  for (uint32_t s = 0; s < j->view->shapes; s++)
  {
    while (at < j->scan_n && j->shape_of[j->order[at]] < s) at++;
    begin[s] = at;
  }
  begin[j->view->shapes] = j->scan_n;
  uint64_t used = persist_off_begin() + (j->view->shapes + 1) * 4;
  P->seq_word[slot] = seq;
  if (!cqlcuda_persistent_copy(P->run, P->params, (uint64_t)slot * P->slot_bytes, sp, used) ||
      !cqlcuda_persistent_copy(P->run, P->ring, (uint64_t)slot * 8, &P->seq_word[slot], 8))
    return 0;
  P->next_seq = seq + 1;
  if (cqlcuda_persistent_running(P->run) != 1 && !persist_launch(P, seq)) return 0;
  /* the answers: poll the done word; a kernel that returned (its idle limit met just before the batch) is
     launched again at this batch, its accumulators cleared */
  struct timespec t0, t;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  uint32_t polls = 0;
  for (;;)
  {
    if (__atomic_load_n(&P->done[slot], __ATOMIC_ACQUIRE) == seq) break;
    if ((++polls & 1023u) == 0)
    {
      int r = cqlcuda_persistent_running(P->run);
      if (__atomic_load_n(&P->done[slot], __ATOMIC_ACQUIRE) == seq) break;
      if (r < 0)
      {
        P->broken = 1;
        snprintf(why, why_cap, "the persistent scan failed: %s", cqlcuda_last_error());
        return 0;
      }
      if (r == 0 && !persist_launch(P, seq)) return 0;
      clock_gettime(CLOCK_MONOTONIC, &t);
      if ((t.tv_sec - t0.tv_sec) * 1000.0 + (t.tv_nsec - t0.tv_nsec) / 1e6 > PERSIST_WAIT_MS)
      {
        P->broken = 1;
        snprintf(why, why_cap, "the persistent scan did not answer batch %llu within %d ms", (unsigned long long)seq, PERSIST_WAIT_MS);
        return 0;
      }
    }
  }
  const uint64_t* ans = P->answers + (uint64_t)slot * CQL_BATCH_LAUNCH_QUERIES * 3;
  for (uint32_t i = 0; i < j->scan_n; i++)
  {
    uint32_t q = j->order[i];
    out_counts[q] = ans[i * 3];
    if (!out_sums) continue;
    if (j->qsum[q] == 0xffffffffu)
    {
      out_sums[q] = 0.0;
      continue;
    }
    double v = (double)(int64_t)ans[i * 3 + 2] * 18446744073709551616.0 + (double)ans[i * 3 + 1];
    out_sums[q] = v / j->col_scale[j->qsum[q]];
  }
  P->batches++;
  return 1;
}

int cqlops_batch_persist_run(CqlBatchPersist* p, const CqlProgram* const* programs, uint32_t query_count, const int32_t* sum_columns,
                             uint64_t* out_counts, double* out_sums)
{
  cqlops_note_error("");
  if (!p) return refuse("no persistent scan");
  if (query_count == 0) return 1;
  pthread_mutex_lock(&p->lock);
  tl_persist = p;
  int ok = batch_run(p->catalog, programs, query_count, p->columns, p->column_count, sum_columns, p->rows_per_thread, out_counts, out_sums,
                     NULL, BATCH_PERSIST, NULL, 0, NULL, 0);
  tl_persist = NULL;
  pthread_mutex_unlock(&p->lock);
  return ok;
}

void cqlops_batch_persist_stats(CqlBatchPersist* p, uint64_t* out_batches, uint64_t* out_launches, uint64_t* out_compiles)
{
  if (out_batches) *out_batches = p ? p->batches : 0;
  if (out_launches) *out_launches = p ? p->launches : 0;
  if (out_compiles) *out_compiles = p ? p->compiles : 0;
}

uint32_t cqlops_batch_persist_ctas(CqlBatchPersist* p)
{
  return p && p->run ? cqlcuda_persistent_ctas(p->run) : 0;
}

int cqlops_batch_persist_destroy(CqlBatchPersist* p)
{
  if (!p) return 1;
  pthread_mutex_lock(&p->lock);
  int ok = persist_stop(p);
  pthread_mutex_unlock(&p->lock);
  if (!ok) return 0;   /* still running: nothing is freed under it */
  cqlcuda_buffer_release(p->ring);
  cqlcuda_buffer_release(p->params);
  cqlcuda_buffer_release(p->state);
  cqlcuda_buffer_release(p->answers_buf);
  free(p->staging);
  pthread_mutex_destroy(&p->lock);
  free(p);
  return 1;
}

/* ---- the autotuner ----
   With rows_per_thread = CQLOPS_BATCH_AUTOTUNE the form of the shared scan is picked per plan shape from
   timed runs: the first batches of a shape run once in each candidate form (the register form with 4, 8
   or 16 rows a thread and 256 or 512 threads a CTA, and the shared-memory tile form), each compiled before
   its run is timed; later batches of the shape run in the fastest. Every form gives the same answers (one
   summand scale for all forms), so the trial runs are ordinary batches. A plan shape is the queries'
   bytecode (literals apart) and summed columns, the column types, the query count and the table's rows,
   each of the last two to a power of two; with a catalog, the catalog and the shapes it holds. The
   reference builds its shared scans from spec-constant modules chosen by fixed rules
   (src/query_exec/query_kernel.c:1782-2041); here the choice is measured on the device that runs it. */

#define BATCH_TUNE_ENTRIES 256
static const uint32_t g_tune_forms[] = { 4u | (1u << 8), 8u | (1u << 8), 16u | (1u << 8), 8u | (2u << 8), 16u | (2u << 8), 0u };
#define BATCH_TUNE_FORMS (sizeof(g_tune_forms) / sizeof(g_tune_forms[0]))
#define BATCH_DEFAULT_FORM (4u | (1u << 8))

typedef struct
{
  uint64_t key;
  uint32_t next;       /* the candidate to time next; BATCH_TUNE_FORMS once tuned */
  uint32_t busy;       /* a thread is timing a candidate */
  uint32_t best;
  double ms[BATCH_TUNE_FORMS];
  uint64_t last_use;
} TuneEntry;

static TuneEntry g_tune[BATCH_TUNE_ENTRIES];
static uint32_t g_tune_count;
static uint64_t g_tune_clock;
static pthread_mutex_t g_tune_lock = PTHREAD_MUTEX_INITIALIZER;
static __thread uint32_t tl_last_form;

static uint64_t tune_mix(uint64_t h, uint64_t v)
{
  for (int i = 0; i < 8; i++) h = (h ^ ((v >> (8 * i)) & 0xffu)) * 1099511628211ull;
  return h;
}

static uint32_t log2_floor(uint64_t v)
{
  uint32_t r = 0;
  while (v >>= 1) r++;
  return r;
}

static uint64_t tune_key(CqlBatchCatalog* catalog, const CqlProgram* const* programs, uint32_t query_count, const CqlColumn* columns,
                         uint32_t column_count, const int32_t* sum_columns)
{
  uint64_t h = 1469598103934665603ull;
  h = tune_mix(h, log2_floor(query_count));
  h = tune_mix(h, log2_floor(columns[0].rows ? columns[0].rows : 1));
  for (uint32_t c = 0; c < column_count; c++) h = tune_mix(h, columns[c].type);
  if (catalog)
  {
    h = tune_mix(h, (uint64_t)(uintptr_t)catalog);
    h = tune_mix(h, cqlops_batch_catalog_shapes(catalog));
    return h;
  }
  for (uint32_t q = 0; q < query_count; q++)
  {
    const CqlProgram* p = programs[q];
    h = tune_mix(h, p->word_count);
    for (uint32_t w = 0; w < p->word_count; w++) h = tune_mix(h, p->words[w]);
    h = tune_mix(h, (uint64_t)(int64_t)(sum_columns ? sum_columns[q] : -1));
  }
  return h;
}

static double now_ms(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec * 1e3 + (double)ts.tv_nsec * 1e-6;
}

static int batch_autotuned(CqlBatchCatalog* catalog, const CqlProgram* const* programs, uint32_t query_count, const CqlColumn* columns,
                           uint32_t column_count, const int32_t* sum_columns, uint64_t* out_counts, double* out_sums, uint32_t* out_shapes)
{
  uint64_t key = tune_key(catalog, programs, query_count, columns, column_count, sum_columns);
  pthread_mutex_lock(&g_tune_lock);
  TuneEntry* e = NULL;
  for (uint32_t i = 0; i < g_tune_count && !e; i++)
    if (g_tune[i].key == key) e = &g_tune[i];
  if (!e)
  {
    uint32_t slot = g_tune_count;
    if (slot < BATCH_TUNE_ENTRIES) g_tune_count++;
    else
    {
      slot = 0;
      for (uint32_t i = 1; i < BATCH_TUNE_ENTRIES; i++)
        if (!g_tune[i].busy && (g_tune[slot].busy || g_tune[i].last_use < g_tune[slot].last_use)) slot = i;
    }
    e = &g_tune[slot];
    memset(e, 0, sizeof(*e));
    e->key = key;
  }
  e->last_use = ++g_tune_clock;
  int trial = e->next < BATCH_TUNE_FORMS && !e->busy;
  uint32_t candidate = e->next;
  uint32_t form = trial ? g_tune_forms[candidate] : (e->next >= BATCH_TUNE_FORMS ? g_tune_forms[e->best] : BATCH_DEFAULT_FORM);
  if (trial) e->busy = 1;
  pthread_mutex_unlock(&g_tune_lock);

  int ok;
  if (trial)
  {
    /* the candidate's kernel is compiled (and the catalog's shapes entered) before the clock starts */
    ok = batch_run(catalog, programs, query_count, columns, column_count, sum_columns, form, NULL, NULL, NULL, BATCH_PREPARE, NULL, 0,
                   NULL, 1);
    double t0 = now_ms();
    ok = ok && batch_run(catalog, programs, query_count, columns, column_count, sum_columns, form, out_counts, out_sums, out_shapes, BATCH_RUN,
                         NULL, 0, NULL, 1);
    double dt = now_ms() - t0;
    pthread_mutex_lock(&g_tune_lock);
    /* the entry may have been taken for another shape meanwhile: record only into this shape's */
    if (e->key == key && e->busy && e->next == candidate)
    {
      e->ms[candidate] = ok ? dt : 1e300;
      e->next = candidate + 1;
      if (e->next == BATCH_TUNE_FORMS)
      {
        uint32_t best = 0;
        for (uint32_t i = 1; i < BATCH_TUNE_FORMS; i++)
          if (e->ms[i] < e->ms[best]) best = i;
        e->best = best;
      }
      e->busy = 0;
    }
    pthread_mutex_unlock(&g_tune_lock);
  }
  else
    ok = batch_run(catalog, programs, query_count, columns, column_count, sum_columns, form, out_counts, out_sums, out_shapes, BATCH_RUN,
                   NULL, 0, NULL, 1);
  tl_last_form = form | (trial ? 1u << 16 : 0u);
  return ok;
}

uint32_t cqlops_batch_last_form(void)
{
  return tl_last_form;
}

void cqlops_batch_tuner_reset(void)
{
  pthread_mutex_lock(&g_tune_lock);
  g_tune_count = 0;
  memset(g_tune, 0, sizeof(g_tune));
  pthread_mutex_unlock(&g_tune_lock);
}

int cqlops_batch_filter_aggregate(const CqlProgram* const* programs, uint32_t query_count, const CqlColumn* columns, uint32_t column_count,
                                  const int32_t* sum_columns, uint32_t rows_per_thread, uint64_t* out_counts, double* out_sums,
                                  uint32_t* out_shapes)
{
  if (rows_per_thread == CQLOPS_BATCH_AUTOTUNE && query_count)
    return batch_autotuned(NULL, programs, query_count, columns, column_count, sum_columns, out_counts, out_sums, out_shapes);
  tl_last_form = rows_per_thread;
  return batch_run(NULL, programs, query_count, columns, column_count, sum_columns, rows_per_thread, out_counts, out_sums, out_shapes,
                   BATCH_RUN, NULL, 0, NULL, 1);
}

int cqlops_batch_filter_aggregate_cat(CqlBatchCatalog* catalog, const CqlProgram* const* programs, uint32_t query_count,
                                      const CqlColumn* columns, uint32_t column_count, const int32_t* sum_columns, uint32_t rows_per_thread,
                                      uint64_t* out_counts, double* out_sums, uint32_t* out_shapes)
{
  if (rows_per_thread == CQLOPS_BATCH_AUTOTUNE && query_count)
    return batch_autotuned(catalog, programs, query_count, columns, column_count, sum_columns, out_counts, out_sums, out_shapes);
  tl_last_form = rows_per_thread;
  return batch_run(catalog, programs, query_count, columns, column_count, sum_columns, rows_per_thread, out_counts, out_sums, out_shapes,
                   BATCH_RUN, NULL, 0, NULL, 1);
}

int cqlops_batch_prepare(CqlBatchCatalog* catalog, const CqlProgram* const* programs, uint32_t query_count, const CqlColumn* columns,
                         uint32_t column_count, const int32_t* sum_columns, uint32_t rows_per_thread)
{
  if (rows_per_thread == CQLOPS_BATCH_AUTOTUNE) rows_per_thread = BATCH_DEFAULT_FORM;
  return batch_run(catalog, programs, query_count, columns, column_count, sum_columns, rows_per_thread, NULL, NULL, NULL, BATCH_PREPARE,
                   NULL, 0, NULL, 1);
}

int cqlops_batch_source(const CqlProgram* const* programs, uint32_t query_count, const CqlColumn* columns, uint32_t column_count,
                        const int32_t* sum_columns, uint32_t rows_per_thread, char* out, uint64_t cap, uint64_t* out_len, uint32_t* out_shapes)
{
  if (rows_per_thread == CQLOPS_BATCH_AUTOTUNE) rows_per_thread = BATCH_DEFAULT_FORM;
  return batch_run(NULL, programs, query_count, columns, column_count, sum_columns, rows_per_thread, NULL, NULL, out_shapes, BATCH_SOURCE, out,
                   cap, out_len, 0);
}

int cqlops_batch_cube_source(const CqlProgram* const* programs, uint32_t query_count, const CqlColumn* columns, uint32_t column_count,
                             const int32_t* sum_columns, uint32_t which, char* out, uint64_t cap, uint64_t* out_len, uint32_t* out_cube_queries)
{
  return batch_run(NULL, programs, query_count, columns, column_count, sum_columns, which ? which - 1 : 0, NULL, NULL, out_cube_queries,
                   which ? BATCH_CUBE_BUILD_SOURCE : BATCH_CUBE_ANSWER_SOURCE, out, cap, out_len, 1);
}
