// Scan + filter kernels.
//
//  scan_simple - contract of src/gpu/vulkan/shaders/scan_simple.comp:1-383: an AND of up to 8 numeric
//                comparisons, 8 rows per thread, leaf words laid out by qe_simple_leaf_words
//                (src/query_exec/query_exec.c:1443-1460) and qe_scan_int_leaf_words (:1407-1440).
//
// GB300 design: a persistent grid; every thread evaluates 8 consecutive rows with 16-byte loads
// (32 bytes of a u32 column in flight per thread), the match bits are compacted with a warp
// prefix sum of popc() and one global atomic per CTA and pass. When the output binding has no room
// for a single row (a COUNT(*) with no row list) every CTA counts privately and adds once at the end.
// When rows are wanted, the scans write a bitmap of the table's rows instead (bitmap mode): every
// 32-row word is stored once by the lanes that evaluated it, with no atomics and no capacity, and the
// bitmap becomes ascending rows on the device (cql_bitmap_popc, prefix_sum, cql_bitmap_emit) - the
// reference's list, unordered across workgroups, had to be sorted on the host.
#include "cql_internal.cuh"
#include <math_constants.h>
#include <climits>
#include <algorithm>

#define COLTYPE_U32 1u
#define COLTYPE_F32 3u
#define COLTYPE_F64 4u
#define COLTYPE_I32 7u

#define CMP_EQ 0u
#define CMP_LT 1u
#define CMP_LE 2u
#define CMP_GT 3u
#define CMP_GE 4u

#define SCAN_INT_FLAG  0x10000u
#define SCAN_INT_NEVER 0x20000u
#define SCAN_INT_BIAS  0x40000u

#define SCAN_THREADS 256
#define ROWS_PER_THREAD 8u

struct Leaf
{
  uint32_t slot, coltype, width, flags, op, w3, w4, enc_base;
};

__device__ __forceinline__ double widen_word(uint32_t coltype, uint32_t word)
{
  if (coltype == COLTYPE_U32) return (double)word;
  if (coltype == COLTYPE_I32) return (double)(int)word;
  return (double)__uint_as_float(word);
}

__device__ __forceinline__ bool cmp(uint32_t op, double v, double t)
{
  switch (op)
  {
    case CMP_EQ: return v == t;
    case CMP_LT: return v < t;
    case CMP_LE: return v <= t;
    case CMP_GT: return v > t;
    default: return v >= t;
  }
}

// Bits of `valid` rows starting at first_row (a multiple of 8) for one integer-interval leaf.
__device__ __forceinline__ uint32_t leaf_int_bits(const Leaf& L, const uint32_t* col, uint64_t first_row, uint32_t valid, uint32_t chunk_start)
{
  uint32_t lo = L.w3, span = L.w4;
  uint32_t bias = (L.flags & SCAN_INT_BIAS) ? 0x80000000u : 0u;
  uint32_t bits = 0;
  if (L.width == 3)
  {
    for (uint32_t k = 0; k < valid; k++) bits |= ((chunk_start + (uint32_t)first_row + k - lo) <= span ? 1u : 0u) << k;
    return bits;
  }
  if (valid == ROWS_PER_THREAD)
  {
    if (L.width == 1)
    {
      uint2 w = *(const uint2*)(col + first_row / 4);
#pragma unroll
      for (uint32_t k = 0; k < 4; k++)
      {
        bits |= ((((w.x >> (k * 8)) & 0xffu) - lo) <= span ? 1u : 0u) << k;
        bits |= ((((w.y >> (k * 8)) & 0xffu) - lo) <= span ? 1u : 0u) << (k + 4);
      }
      return bits;
    }
    if (L.width == 2)
    {
      uint4 w = __ldcs((const uint4*)(col + first_row / 2));
      uint32_t ws[4] = { w.x, w.y, w.z, w.w };
#pragma unroll
      for (uint32_t k = 0; k < 4; k++)
      {
        bits |= (((ws[k] & 0xffffu) - lo) <= span ? 1u : 0u) << (2 * k);
        bits |= (((ws[k] >> 16) - lo) <= span ? 1u : 0u) << (2 * k + 1);
      }
      return bits;
    }
    const uint4* v = (const uint4*)(col + first_row);
    uint4 a = __ldcs(v), b = __ldcs(v + 1);
    uint32_t ws[8] = { a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w };
#pragma unroll
    for (uint32_t k = 0; k < 8; k++) bits |= (((ws[k] ^ bias) - lo) <= span ? 1u : 0u) << k;
    return bits;
  }
  for (uint32_t k = 0; k < valid; k++)
  {
    uint64_t row = first_row + k;
    uint32_t code;
    if (L.width == 1) code = (col[row >> 2] >> ((row & 3) * 8)) & 0xffu;
    else if (L.width == 2) code = (col[row >> 1] >> ((row & 1) * 16)) & 0xffffu;
    else code = col[row] ^ bias;
    bits |= ((code - lo) <= span ? 1u : 0u) << k;
  }
  return bits;
}

// Bits for a leaf compared in double, as compare_rows in scan_simple.comp does.
__device__ __forceinline__ uint32_t leaf_f64_bits(const Leaf& L, const uint32_t* col, uint64_t first_row, uint32_t valid)
{
  double target = __hiloint2double((int)L.w4, (int)L.w3);
  uint32_t bits = 0;
  uint32_t op = L.op;
  if (valid == ROWS_PER_THREAD && L.width == 1)
  {
    uint2 w = *(const uint2*)(col + first_row / 4);
#pragma unroll
    for (uint32_t k = 0; k < 4; k++)
    {
      bits |= (cmp(op, widen_word(L.coltype, L.enc_base + ((w.x >> (k * 8)) & 0xffu)), target) ? 1u : 0u) << k;
      bits |= (cmp(op, widen_word(L.coltype, L.enc_base + ((w.y >> (k * 8)) & 0xffu)), target) ? 1u : 0u) << (k + 4);
    }
    return bits;
  }
  if (valid == ROWS_PER_THREAD && L.width == 2)
  {
    uint4 w = __ldcs((const uint4*)(col + first_row / 2));
    uint32_t ws[4] = { w.x, w.y, w.z, w.w };
#pragma unroll
    for (uint32_t k = 0; k < 4; k++)
    {
      bits |= (cmp(op, widen_word(L.coltype, L.enc_base + (ws[k] & 0xffffu)), target) ? 1u : 0u) << (2 * k);
      bits |= (cmp(op, widen_word(L.coltype, L.enc_base + (ws[k] >> 16)), target) ? 1u : 0u) << (2 * k + 1);
    }
    return bits;
  }
  if (valid == ROWS_PER_THREAD)
  {
    if (L.coltype == COLTYPE_F64)
    {
      const uint4* v = (const uint4*)(col + first_row * 2);
#pragma unroll
      for (uint32_t q = 0; q < 4; q++)
      {
        uint4 w = __ldcs(v + q);
        double a = __hiloint2double((int)w.y, (int)w.x);
        double b = __hiloint2double((int)w.w, (int)w.z);
        bits |= (cmp(op, a, target) ? 1u : 0u) << (2 * q);
        bits |= (cmp(op, b, target) ? 1u : 0u) << (2 * q + 1);
      }
      return bits;
    }
    const uint4* v = (const uint4*)(col + first_row);
    uint4 a = __ldcs(v), b = __ldcs(v + 1);
    uint32_t ws[8] = { a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w };
#pragma unroll
    for (uint32_t k = 0; k < 8; k++) bits |= (cmp(op, widen_word(L.coltype, ws[k]), target) ? 1u : 0u) << k;
    return bits;
  }
  for (uint32_t k = 0; k < valid; k++)
  {
    uint64_t row = first_row + k;
    double value;
    if (L.width == 1) value = widen_word(L.coltype, L.enc_base + ((col[row >> 2] >> ((row & 3) * 8)) & 0xffu));
    else if (L.width == 2) value = widen_word(L.coltype, L.enc_base + ((col[row >> 1] >> ((row & 1) * 16)) & 0xffffu));
    else if (L.coltype == COLTYPE_F64) value = ((const double*)col)[row];
    else value = widen_word(L.coltype, col[row]);
    bits |= (cmp(op, value, target) ? 1u : 0u) << k;
  }
  return bits;
}

template <bool COUNT_ONLY>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_simple(CqlLaunch a, uint64_t rows)
{
  __shared__ Leaf s_leaf[8];
  __shared__ uint32_t s_leaf_count;
  __shared__ uint32_t s_warp_total[SCAN_THREADS / 32];
  __shared__ uint32_t s_base;

  const uint32_t* leaf_words = (const uint32_t*)a.buf[0];
  if (threadIdx.x == 0)
  {
    uint32_t n = leaf_words[0];
    s_leaf_count = n > 8 ? 8 : n;
  }
  __syncthreads();
  if (threadIdx.x < s_leaf_count)
  {
    const uint32_t* w = leaf_words + 1 + threadIdx.x * 6;
    Leaf L;
    L.slot = w[0];
    L.coltype = w[1] & 0xffu;
    L.width = (w[1] >> 8) & 0xffu;
    L.flags = w[1] & 0x70000u;
    L.op = w[2];
    L.w3 = w[3];
    L.w4 = w[4];
    L.enc_base = w[5];
    s_leaf[threadIdx.x] = L;
  }
  __syncthreads();

  uint32_t* out = (uint32_t*)a.buf[3];
  uint32_t* out_count = (uint32_t*)a.buf[4];
  const uint32_t* skip = (const uint32_t*)a.buf[5];
  uint64_t capacity = a.bytes[3] / 8;
  uint32_t skip_shift = cql_word(a, 6);
  bool skip_on = cql_word(a, 8) != 0;
  uint32_t chunk_start = cql_word(a, 10);
  uint32_t row_offset = cql_word(a, 12);   // added to every row written (a dispatch over one range of the table)
  // word 14: 1 = the matches as a bitmap of the table's rows from row word 2 on (binding 3, one bit a row,
  // each 32-row word written by the four lanes that own it; the dispatch's first row is a multiple of 32)
  const bool bitmap_mode = !COUNT_ONLY && cql_word(a, 14) != 0;
  const uint64_t bitmap_words = a.bytes[3] / 4;
  const uint32_t bitmap_first = cql_word(a, 2);   // the table row of the bitmap's first bit (a multiple of 32)
  uint32_t leaf_count = s_leaf_count;

  uint64_t groups = (rows + ROWS_PER_THREAD - 1) / ROWS_PER_THREAD;
  uint64_t per_pass = (uint64_t)gridDim.x * SCAN_THREADS;
  uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t private_count = 0;

  // COUNT(*) of one whole-number comparison on a full-width column (the common count query): 16 rows
  // per thread with all four 16-byte loads issued before the compares, twice the bytes in flight of the
  // general loop. The condition is the same for every thread of the grid.
  const Leaf& L0 = s_leaf[0];
  if (COUNT_ONLY && leaf_count == 1 && (L0.flags & SCAN_INT_FLAG) && !(L0.flags & SCAN_INT_NEVER) && L0.width == 0 && !skip_on)
  {
    const uint32_t* col = (const uint32_t*)a.buf[6 + (L0.slot < 10 ? L0.slot : 0)];
    const uint32_t lo = L0.w3, span = L0.w4, bias = (L0.flags & SCAN_INT_BIAS) ? 0x80000000u : 0u;
    const uint64_t blocks16 = rows / 16;
    for (uint64_t g = (uint64_t)blockIdx.x * SCAN_THREADS + threadIdx.x; g < blocks16; g += per_pass)
    {
      const uint4* v = (const uint4*)(col + g * 16);
      uint4 q0 = __ldcs(v), q1 = __ldcs(v + 1), q2 = __ldcs(v + 2), q3 = __ldcs(v + 3);
      uint32_t w[16] = { q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x, q2.y, q2.z, q2.w, q3.x, q3.y, q3.z, q3.w };
#pragma unroll
      for (uint32_t k = 0; k < 16; k++) private_count += ((w[k] ^ bias) - lo) <= span ? 1u : 0u;
    }
    for (uint64_t r = blocks16 * 16 + (uint64_t)blockIdx.x * SCAN_THREADS + threadIdx.x; r < rows; r += per_pass)
      private_count += ((col[r] ^ bias) - lo) <= span ? 1u : 0u;
    groups = 0;   // the general loop below has nothing left to do
  }

  for (uint64_t base_group = (uint64_t)blockIdx.x * SCAN_THREADS; base_group < groups; base_group += per_pass)
  {
    uint64_t g = base_group + threadIdx.x;
    uint64_t first_row = g * ROWS_PER_THREAD;
    uint32_t valid = first_row < rows ? (uint32_t)min((uint64_t)ROWS_PER_THREAD, rows - first_row) : 0u;
    uint32_t live = valid == 0 ? 0u : ((1u << valid) - 1u);
    if (live && skip_on)
    {
      uint64_t chunk = first_row >> skip_shift;
      if (skip[chunk >> 5] & (1u << (chunk & 31))) live = 0;
    }
    for (uint32_t l = 0; l < leaf_count && live; l++)
    {
      const Leaf& L = s_leaf[l];
      const uint32_t* col = (const uint32_t*)a.buf[6 + (L.slot < 10 ? L.slot : 0)];
      if (L.flags & SCAN_INT_FLAG)
      {
        if (L.flags & SCAN_INT_NEVER) live = 0;
        else live &= leaf_int_bits(L, col, first_row, valid, chunk_start);
      }
      else
      {
        live &= leaf_f64_bits(L, col, first_row, valid);
      }
    }
    uint32_t n = __popc(live);
    if (COUNT_ONLY)
    {
      private_count += n;
      continue;
    }
    if (bitmap_mode)
    {
      // eight rows a lane, four lanes a 32-row word; every word of the dispatch written once
      uint32_t m = live << (8u * (lane & 3u));
      m |= __shfl_xor_sync(0xffffffffu, m, 1);
      m |= __shfl_xor_sync(0xffffffffu, m, 2);
      uint64_t word = ((uint64_t)(row_offset - bitmap_first) >> 5) + (g >> 2);
      if ((lane & 3u) == 0u && word < bitmap_words) out[word] = m;
      private_count += n;
      continue;
    }
    // warp inclusive scan of the match counts
    uint32_t incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) s_warp_total[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0)
    {
      uint32_t run = 0;
      for (int w = 0; w < SCAN_THREADS / 32; w++)
      {
        uint32_t t = s_warp_total[w];
        s_warp_total[w] = run;
        run += t;
      }
      s_base = run ? atomicAdd(out_count, run) : 0u;
    }
    __syncthreads();
    uint64_t pos = (uint64_t)s_base + s_warp_total[warp] + (incl - n);
    while (live)
    {
      uint32_t k = __ffs(live) - 1;
      live &= live - 1;
      if (pos < capacity)
      {
        uint2 pair = make_uint2(row_offset + (uint32_t)(first_row + k), 0u);
        *(uint2*)(out + pos * 2) = pair;
      }
      pos++;
    }
    __syncthreads();
  }
  if (COUNT_ONLY || bitmap_mode)
  {
    uint32_t w = private_count;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
    if (lane == 0) s_warp_total[warp] = w;
    __syncthreads();
    if (threadIdx.x == 0)
    {
      uint32_t total = 0;
      for (int i = 0; i < SCAN_THREADS / 32; i++) total += s_warp_total[i];
      if (total) atomicAdd(out_count, total);
    }
  }
}

static int launch_scan_simple(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = cql_word(a, 0);
  if (rows == 0) return 0;
  uint64_t groups = (rows + ROWS_PER_THREAD - 1) / ROWS_PER_THREAD;
  uint64_t ctas = (groups + SCAN_THREADS - 1) / SCAN_THREADS;
  uint32_t grid = cql_stream_grid(ctas, 8);
  // no room for one row pair and no bitmap: count only (a bitmap of at most 32 rows is one 4-byte word)
  bool count_only = a.bytes[3] < 8 && cql_word(a, 14) == 0;
  if (count_only) k_scan_simple<true><<<grid, SCAN_THREADS, 0, stream>>>(a, rows);
  else k_scan_simple<false><<<grid, SCAN_THREADS, 0, stream>>>(a, rows);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// scan_filter - the bytecode interpreter (contract of src/gpu/vulkan/shaders/scan_filter.comp:1-559):
// opcodes of src/query_exec/query_exec.h:58-81 over a double stack of 8, one row per thread, the
// instruction pointer and the step count bounded by the program length. It runs only for shapes a
// per-query kernel could not be built for. Trigram similarity and edit distance are not evaluated
// The fuzzy comparisons SIMILARITY (trigram similarity) and EDIT_DISTANCE (scan_filter.comp:236-323)
// leave their score in the output pair's second word (an f32 similarity, an integer distance) when
// word 2 has bit 0; word 4 is the gram length.

#define IOP_PUSH_TRUE 0
#define IOP_LOAD_NUM_COL 1
#define IOP_PUSH_CONST 2
#define IOP_CMP_EQ 3
#define IOP_CMP_NE 4
#define IOP_CMP_LT 5
#define IOP_CMP_GT 6
#define IOP_CMP_LE 7
#define IOP_CMP_GE 8
#define IOP_AND 9
#define IOP_OR 10
#define IOP_STR_EQ 11
#define IOP_STR_CONTAINS 12
#define IOP_HALT 13
#define IOP_PUSH_FALSE 14
#define IOP_TRIGRAM_SIM 15
#define IOP_EDIT_DISTANCE 16
#define IOP_STR_NE 17
#define IOP_STR_LT 18
#define IOP_STR_GT 19
#define IOP_STR_LE 20
#define IOP_STR_GE 21
#define INTERP_MAX_STACK 8

__device__ __forceinline__ const uint32_t* slot_words(const CqlLaunch& a, uint32_t slot) { return (const uint32_t*)a.buf[6 + (slot < 10 ? slot : 0)]; }

__device__ double interp_load(const CqlLaunch& a, uint32_t slot, uint32_t coltype, uint64_t row)
{
  const uint32_t* w = slot_words(a, slot);
  switch (coltype)
  {
    case 1: case 12: return (double)w[row];
    case 2: return (double)w[row * 2 + 1] * 4294967296.0 + (double)w[row * 2];
    case 3: return (double)__uint_as_float(w[row]);
    case 4: return __hiloint2double((int)w[row * 2 + 1], (int)w[row * 2]);
    case 6: return (double)((const unsigned char*)w)[row];
    case 7: case 9: return (double)(int)w[row];
    default:
    {
      uint32_t lo = w[row * 2], hi = w[row * 2 + 1];
      double u = (double)hi * 4294967296.0 + (double)lo;
      return (hi & 0x80000000u) ? u - 18446744073709551616.0 : u;
    }
  }
}

__device__ __forceinline__ uint32_t str_off(const CqlLaunch& a, uint32_t slot, uint64_t row) { return slot_words(a, slot + 1)[row * 2]; }
__device__ __forceinline__ uint32_t str_byte(const CqlLaunch& a, uint32_t slot, uint64_t i) { return ((const unsigned char*)slot_words(a, slot))[i]; }
__device__ __forceinline__ uint32_t const_byte(const CqlLaunch& a, uint32_t wo, uint32_t i) { return ((const unsigned char*)a.buf[2])[wo * 4u + i]; }

__device__ int interp_str_cmp3(const CqlLaunch& a, uint32_t slot, uint64_t row, uint32_t wo, uint32_t len)
{
  uint32_t s = str_off(a, slot, row), e = str_off(a, slot, row + 1), n = e - s, m = n < len ? n : len;
  for (uint32_t i = 0; i < m; i++)
  {
    uint32_t x = str_byte(a, slot, s + i), y = const_byte(a, wo, i);
    if (x != y) return x < y ? -1 : 1;
  }
  return n < len ? -1 : (n > len ? 1 : 0);
}

__device__ bool interp_str_contains(const CqlLaunch& a, uint32_t slot, uint64_t row, uint32_t wo, uint32_t len)
{
  uint32_t s = str_off(a, slot, row), e = str_off(a, slot, row + 1), n = e - s;
  if (len == 0) return true;
  if (n < len) return false;
  for (uint32_t i = 0; i + len <= n; i++)
  {
    uint32_t j = 0;
    while (j < len && str_byte(a, slot, s + i + j) == const_byte(a, wo, j)) j++;
    if (j == len) return true;
  }
  return false;
}

#define FUZZY_MAX_NEEDLE 64u          // QE_FUZZY_MAX_NEEDLE_LEN, scan_filter.comp:35
#define FUZZY_MAX_STRING 1048576u     // MAX_SANE_STRING_LEN, scan_filter.comp:205

// the shared n-grams of the row and the needle (each needle gram used once, the first unused match taken)
// over the union of the two gram counts
__device__ double interp_trigram(const CqlLaunch& a, uint32_t slot, uint64_t row, uint32_t wo, uint32_t clen, uint32_t n)
{
  uint32_t s = str_off(a, slot, row), e = str_off(a, slot, row + 1), len = e - s;
  if (len < n || clen < n)
  {
    if (len != clen) return 0.0;
    for (uint32_t i = 0; i < len; i++)
      if (str_byte(a, slot, s + i) != const_byte(a, wo, i)) return 0.0;
    return 1.0;
  }
  if (len > FUZZY_MAX_STRING) return 0.0;
  uint32_t needle_grams = min(clen - n + 1u, FUZZY_MAX_NEEDLE);
  unsigned long long used = 0ull;   // one bit per needle gram (at most 64)
  uint32_t shared = 0;
  for (uint32_t i = 0; i + n <= len; i++)
    for (uint32_t j = 0; j < needle_grams; j++)
    {
      if ((used >> j) & 1ull) continue;
      uint32_t k = 0;
      while (k < n && str_byte(a, slot, s + i + k) == const_byte(a, wo, j + k)) k++;
      if (k == n)
      {
        used |= 1ull << j;
        shared++;
        break;
      }
    }
  uint32_t uni = (len - n + 1u) + needle_grams - shared;
  return uni == 0 ? 0.0 : (double)shared / (double)uni;
}

// the Levenshtein distance to the first 64 bytes of the needle, one rolling row
__device__ double interp_edit_distance(const CqlLaunch& a, uint32_t slot, uint64_t row, uint32_t wo, uint32_t clen)
{
  uint32_t s = str_off(a, slot, row), e = str_off(a, slot, row + 1), len = e - s;
  if (len > FUZZY_MAX_STRING) return (double)FUZZY_MAX_STRING;
  uint32_t m = min(clen, FUZZY_MAX_NEEDLE);
  uint32_t dp[FUZZY_MAX_NEEDLE + 1];
  for (uint32_t j = 0; j <= m; j++) dp[j] = j;
  for (uint32_t i = 1; i <= len; i++)
  {
    uint32_t diag = dp[0];
    dp[0] = i;
    uint32_t hb = str_byte(a, slot, s + i - 1);
    for (uint32_t j = 1; j <= m; j++)
    {
      uint32_t keep = dp[j];
      uint32_t cost = hb == const_byte(a, wo, j - 1) ? 0u : 1u;
      dp[j] = min(min(dp[j] + 1u, dp[j - 1] + 1u), diag + cost);
      diag = keep;
    }
  }
  return (double)dp[m];
}

__device__ bool interp_row(const CqlLaunch& a, const uint32_t* code, uint32_t words, uint64_t row, uint32_t gram, uint32_t* aux)
{
  const uint32_t* consts = (const uint32_t*)a.buf[1];
  double stack[INTERP_MAX_STACK];
  int sp = 0;
  uint32_t ip = 0, steps = 0;
  while (ip < words && steps < words + 64u)
  {
    steps++;
    uint32_t op = code[ip++];
    if (op == IOP_HALT) break;
    if (op == IOP_PUSH_TRUE || op == IOP_PUSH_FALSE)
    {
      if (sp >= INTERP_MAX_STACK) return false;
      stack[sp++] = op == IOP_PUSH_TRUE ? 1.0 : 0.0;
    }
    else if (op == IOP_LOAD_NUM_COL)
    {
      if (sp >= INTERP_MAX_STACK || ip >= words) return false;
      uint32_t operand = code[ip++];
      stack[sp++] = interp_load(a, operand & 0xffu, (operand >> 8) & 0xffu, row);
    }
    else if (op == IOP_PUSH_CONST)
    {
      if (sp >= INTERP_MAX_STACK || ip >= words) return false;
      uint32_t k = code[ip++];
      stack[sp++] = __hiloint2double((int)consts[k * 2 + 1], (int)consts[k * 2]);
    }
    else if (op >= IOP_CMP_EQ && op <= IOP_OR)
    {
      if (sp < 2) return false;
      double b = stack[--sp], x = stack[--sp];
      bool r;
      switch (op)
      {
        case IOP_CMP_EQ: r = x == b; break;
        case IOP_CMP_NE: r = x != b; break;
        case IOP_CMP_LT: r = x < b; break;
        case IOP_CMP_GT: r = x > b; break;
        case IOP_CMP_LE: r = x <= b; break;
        case IOP_CMP_GE: r = x >= b; break;
        case IOP_AND: r = x != 0.0 && b != 0.0; break;
        default: r = x != 0.0 || b != 0.0; break;
      }
      stack[sp++] = r ? 1.0 : 0.0;
    }
    else if (op == IOP_STR_EQ || op == IOP_STR_NE || op == IOP_STR_CONTAINS || (op >= IOP_STR_LT && op <= IOP_STR_GE))
    {
      if (sp >= INTERP_MAX_STACK || ip + 3 > words) return false;
      uint32_t slot = code[ip], wo = code[ip + 1], len = code[ip + 2];
      ip += 3;
      if (slot + 1 >= 10) return false;
      bool r;
      if (op == IOP_STR_CONTAINS) r = interp_str_contains(a, slot, row, wo, len);
      else
      {
        int c = interp_str_cmp3(a, slot, row, wo, len);
        r = op == IOP_STR_EQ ? c == 0 : op == IOP_STR_NE ? c != 0 : op == IOP_STR_LT ? c < 0 : op == IOP_STR_GT ? c > 0 : op == IOP_STR_LE ? c <= 0 : c >= 0;
      }
      stack[sp++] = r ? 1.0 : 0.0;
    }
    else if (op == IOP_TRIGRAM_SIM || op == IOP_EDIT_DISTANCE)
    {
      if (sp >= INTERP_MAX_STACK || ip + 3 > words) return false;
      uint32_t slot = code[ip], wo = code[ip + 1], len = code[ip + 2];
      ip += 3;
      if (slot + 1 >= 10) return false;
      double v = op == IOP_TRIGRAM_SIM ? interp_trigram(a, slot, row, wo, len, gram) : interp_edit_distance(a, slot, row, wo, len);
      *aux = op == IOP_TRIGRAM_SIM ? __float_as_uint((float)v) : (uint32_t)v;
      stack[sp++] = v;
    }
    else
    {
      // an opcode this kernel does not evaluate ends the program
      break;
    }
  }
  return sp > 0 && stack[sp - 1] != 0.0;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_filter(CqlLaunch a, uint64_t rows)
{
  __shared__ uint32_t s_warp[SCAN_THREADS / 32];
  __shared__ uint32_t s_base;
  const uint32_t* code = (const uint32_t*)a.buf[0];
  uint32_t words = (uint32_t)(a.bytes[0] / 4);
  uint32_t* out = (uint32_t*)a.buf[3];
  uint32_t* out_count = (uint32_t*)a.buf[4];
  const uint32_t* skip = (const uint32_t*)a.buf[5];
  uint64_t capacity = a.bytes[3] / 8;
  uint32_t skip_shift = cql_word(a, 6);
  bool skip_on = cql_word(a, 8) != 0;
  bool scored = (cql_word(a, 2) & 1u) != 0u;
  uint32_t gram = max(cql_word(a, 4), 1u);
  // word 10: 1 = the matches as a bitmap of the rows (binding 3): a warp's 32 rows are one word, its ballot
  const bool bitmap_mode = cql_word(a, 10) != 0 && !scored;
  const uint64_t bitmap_words = a.bytes[3] / 4;
  uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t bitmap_count = 0;
  for (uint64_t base = (uint64_t)blockIdx.x * SCAN_THREADS; base < rows; base += (uint64_t)gridDim.x * SCAN_THREADS)
  {
    uint64_t row = base + threadIdx.x;
    bool in_range = row < rows;
    if (in_range && skip_on)
    {
      uint64_t ch = row >> skip_shift;
      in_range = ((skip[ch >> 5] >> (ch & 31)) & 1u) == 0u;
    }
    uint32_t aux = 0u;
    bool matched = in_range && interp_row(a, code, words, row, gram, &aux);
    uint32_t ballot = __ballot_sync(0xffffffffu, matched);
    if (bitmap_mode)
    {
      uint64_t word = (base >> 5) + warp;
      if (lane == 0 && word < bitmap_words) out[word] = ballot;
      bitmap_count += __popc(ballot);
      continue;
    }
    if (lane == 0) s_warp[warp] = __popc(ballot);
    __syncthreads();
    if (threadIdx.x == 0)
    {
      uint32_t run = 0;
      for (int w = 0; w < SCAN_THREADS / 32; w++)
      {
        uint32_t t = s_warp[w];
        s_warp[w] = run;
        run += t;
      }
      s_base = run ? atomicAdd(out_count, run) : 0u;
    }
    __syncthreads();
    if (matched)
    {
      uint64_t pos = (uint64_t)s_base + s_warp[warp] + __popc(ballot & ((1u << lane) - 1u));
      if (pos < capacity) *(uint2*)(out + pos * 2) = make_uint2((uint32_t)row, scored ? aux : 0u);
    }
    __syncthreads();
  }
  // one atomic a CTA (a warp's would all meet on the one count word)
  if (bitmap_mode)
  {
    __shared__ uint32_t s_count;
    if (threadIdx.x == 0) s_count = 0;
    __syncthreads();
    if (lane == 0 && bitmap_count) atomicAdd(&s_count, bitmap_count);
    __syncthreads();
    if (threadIdx.x == 0 && s_count) atomicAdd(out_count, s_count);
  }
}

static int launch_scan_filter(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = cql_word(a, 0);
  if (rows == 0) return 0;
  uint32_t grid = cql_stream_grid((rows + SCAN_THREADS - 1) / SCAN_THREADS, 8);
  k_scan_filter<<<grid, SCAN_THREADS, 0, stream>>>(a, rows);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// A selection bitmap (one bit a row, as the scans write it in bitmap mode) to its rows in ascending
// order, in blocks of 256 words (8192 rows): cql_bitmap_popc counts each block's rows (binding 0 bitmap,
// 1 counts per block; word 0 words), the prefix_sum kernel turns the block counts into offsets, and
// cql_bitmap_emit ranks each block's words in shared memory and writes their rows from the block's
// offset (binding 0 bitmap, 1 block offsets, 2 rows; word 0 words, word 2 the row of the first bit). No
// atomics and no sort: the order is the bitmap's; the scan in between is over words / 256 counts.

__device__ __forceinline__ uint32_t bitmap_block_exclusive(uint32_t v, uint32_t* s_warp, uint32_t* total)
{
  uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  uint32_t before = 0, all = 0;
  for (uint32_t w = 0; w < SCAN_THREADS / 32; w++)
  {
    uint32_t t = s_warp[w];
    if (w < warp) before += t;
    all += t;
  }
  __syncthreads();
  *total = all;
  return before + incl - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_bitmap_popc(CqlLaunch a, uint64_t words)
{
  __shared__ uint32_t s_warp[SCAN_THREADS / 32];
  const uint32_t* bits = (const uint32_t*)a.buf[0];
  uint32_t* counts = (uint32_t*)a.buf[1];
  uint64_t blocks = (words + SCAN_THREADS - 1) / SCAN_THREADS;
  for (uint64_t b = blockIdx.x; b < blocks; b += gridDim.x)
  {
    uint64_t w = b * SCAN_THREADS + threadIdx.x;
    uint32_t total;
    bitmap_block_exclusive(w < words ? __popc(bits[w]) : 0u, s_warp, &total);
    if (threadIdx.x == 0) counts[b] = total;
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_bitmap_emit(CqlLaunch a, uint64_t words)
{
  __shared__ uint32_t s_warp[SCAN_THREADS / 32];
  const uint32_t* bits = (const uint32_t*)a.buf[0];
  const uint32_t* offsets = (const uint32_t*)a.buf[1];
  uint32_t* rows = (uint32_t*)a.buf[2];
  uint32_t first = cql_word(a, 2);
  uint64_t cap = a.bytes[2] / 4;
  uint64_t blocks = (words + SCAN_THREADS - 1) / SCAN_THREADS;
  for (uint64_t b = blockIdx.x; b < blocks; b += gridDim.x)
  {
    uint64_t w = b * SCAN_THREADS + threadIdx.x;
    uint32_t m = w < words ? bits[w] : 0u, total;
    uint64_t pos = (uint64_t)offsets[b] + bitmap_block_exclusive(__popc(m), s_warp, &total);
    while (m)
    {
      uint32_t bit = (uint32_t)(__ffs(m) - 1);
      m &= m - 1u;
      if (pos < cap) rows[pos] = first + (uint32_t)(w * 32 + bit);
      pos++;
    }
  }
}

static int launch_bitmap_popc(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t words = cql_word(a, 0);
  if (words == 0) return 0;
  uint64_t blocks = (words + SCAN_THREADS - 1) / SCAN_THREADS;
  if (a.bytes[0] < words * 4 || a.bytes[1] < blocks * 4) return (int)cudaErrorInvalidValue;
  k_bitmap_popc<<<cql_stream_grid(blocks, 8), SCAN_THREADS, 0, stream>>>(a, words);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_bitmap_emit(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t words = cql_word(a, 0);
  if (words == 0) return 0;
  uint64_t blocks = (words + SCAN_THREADS - 1) / SCAN_THREADS;
  if (a.bytes[0] < words * 4 || a.bytes[1] < blocks * 4) return (int)cudaErrorInvalidValue;
  k_bitmap_emit<<<cql_stream_grid(blocks, 8), SCAN_THREADS, 0, stream>>>(a, words);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// cql_zone_map: the per-chunk min/max of a column (cql_column_ensure_zone_map, the zone maps
// qe_scan_build_dispatch_ranges prunes with, src/query_exec/query_exec.c:13294-13540). Binding 0 the
// column, 1 out: f64 (min, max) per chunk, min > max for a chunk without values (all NaN);
// words 0 rows, 2 type (U32/I32/F32/F64), 3 width (0 stored, 1/2 narrow codes), 4 narrow base,
// 6 log2 of the chunk rows. One CTA per chunk at a time.

// integer columns (stored, or narrow codes: value = base + code) compare as 64-bit integers, floats as
// floats: no FP64 arithmetic per row
template <int KIND>  // 0 u32, 1 i32, 2 f32, 3 f64
__global__ void __launch_bounds__(SCAN_THREADS) k_zone_map(CqlLaunch a, uint64_t rows, uint64_t chunks)
{
  __shared__ double s_min[SCAN_THREADS / 32], s_max[SCAN_THREADS / 32];
  const void* col = a.buf[0];
  double* out = (double*)a.buf[1];
  uint32_t width = cql_word(a, 3), base = cql_word(a, 4), log2_rows = cql_word(a, 6);
  uint64_t chunk_rows = 1ull << log2_rows;
  for (uint64_t z = blockIdx.x; z < chunks; z += gridDim.x)
  {
    uint64_t start = z * chunk_rows, end = min(start + chunk_rows, rows);
    double lo, hi;
    if (KIND <= 1)
    {
      long long ilo = LLONG_MAX, ihi = LLONG_MIN;
      for (uint64_t r = start + threadIdx.x; r < end; r += SCAN_THREADS)
      {
        uint32_t w = width == 1 ? base + ((const uint8_t*)col)[r] : width == 2 ? base + ((const uint16_t*)col)[r] : ((const uint32_t*)col)[r];
        long long v = KIND == 1 ? (long long)(int)w : (long long)w;
        ilo = min(ilo, v);
        ihi = max(ihi, v);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
      {
        ilo = min(ilo, __shfl_xor_sync(0xffffffffu, ilo, o));
        ihi = max(ihi, __shfl_xor_sync(0xffffffffu, ihi, o));
      }
      lo = ilo == LLONG_MAX ? CUDART_INF : (double)ilo;
      hi = ihi == LLONG_MIN ? -CUDART_INF : (double)ihi;
    }
    else if (KIND == 2)
    {
      float flo = CUDART_INF_F, fhi = -CUDART_INF_F;
      for (uint64_t r = start + threadIdx.x; r < end; r += SCAN_THREADS)
      {
        float v = ((const float*)col)[r];
        flo = fminf(flo, v);   // fminf/fmaxf pass over NaN
        fhi = fmaxf(fhi, v);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
      {
        flo = fminf(flo, __shfl_xor_sync(0xffffffffu, flo, o));
        fhi = fmaxf(fhi, __shfl_xor_sync(0xffffffffu, fhi, o));
      }
      lo = flo;
      hi = fhi;
    }
    else
    {
      lo = CUDART_INF;
      hi = -CUDART_INF;
      for (uint64_t r = start + threadIdx.x; r < end; r += SCAN_THREADS)
      {
        double v = ((const double*)col)[r];
        lo = fmin(lo, v);
        hi = fmax(hi, v);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
      {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
      }
    }
    if ((threadIdx.x & 31u) == 0)
    {
      s_min[threadIdx.x >> 5] = lo;
      s_max[threadIdx.x >> 5] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
      for (int w = 1; w < SCAN_THREADS / 32; w++)
      {
        lo = fmin(lo, s_min[w]);
        hi = fmax(hi, s_max[w]);
      }
      out[z * 2] = lo;
      out[z * 2 + 1] = hi;
    }
    __syncthreads();
  }
}

static int launch_zone_map(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = cql_word(a, 0);
  uint32_t type = cql_word(a, 2), width = cql_word(a, 3), log2_rows = cql_word(a, 6);
  if (rows == 0) return 0;
  if (log2_rows < 3 || log2_rows > 30 || width > 2 || (width && type != COLTYPE_U32 && type != COLTYPE_I32)) return (int)cudaErrorInvalidValue;
  if (type != COLTYPE_U32 && type != COLTYPE_I32 && type != COLTYPE_F32 && type != COLTYPE_F64) return (int)cudaErrorInvalidValue;
  uint64_t elem = width ? width : (type == COLTYPE_F64 ? 8 : 4);
  uint64_t chunks = (rows + (1ull << log2_rows) - 1) >> log2_rows;
  if (a.bytes[0] < rows * elem || a.bytes[1] < chunks * 16) return (int)cudaErrorInvalidValue;
  uint32_t grid = cql_stream_grid(chunks, 8);
  if (type == COLTYPE_U32) k_zone_map<0><<<grid, SCAN_THREADS, 0, stream>>>(a, rows, chunks);
  else if (type == COLTYPE_I32) k_zone_map<1><<<grid, SCAN_THREADS, 0, stream>>>(a, rows, chunks);
  else if (type == COLTYPE_F32) k_zone_map<2><<<grid, SCAN_THREADS, 0, stream>>>(a, rows, chunks);
  else k_zone_map<3><<<grid, SCAN_THREADS, 0, stream>>>(a, rows, chunks);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// cql_batch_fold: the batched scan's per-CTA partials [cta][query] x (count, sum low, sum high) summed
// over the CTAs into [query] x (count, low, high). One CTA per query; its threads take the CTAs in turn and
// the block combines them in a tree. The sums are 128-bit integers, so any order gives the same bits.
// Binding 0 partials, 1 out; word 0 queries, word 2 CTAs.

struct Fold128
{
  unsigned long long c, lo, hi;
};

__device__ __forceinline__ void fold_add(Fold128& a, unsigned long long c, unsigned long long lo, unsigned long long hi)
{
  unsigned long long l2 = a.lo + lo;
  a.hi += hi + (l2 < a.lo ? 1ull : 0ull);
  a.lo = l2;
  a.c += c;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_batch_fold(CqlLaunch a, uint32_t nq, uint32_t ctas)
{
  const unsigned long long* parts = (const unsigned long long*)a.buf[0];
  unsigned long long* out = (unsigned long long*)a.buf[1];
  const uint64_t pcap = a.bytes[0] / 24;
  __shared__ Fold128 s_warp[SCAN_THREADS / 32];
  for (uint32_t q = blockIdx.x; q < nq; q += gridDim.x)
  {
    Fold128 f = { 0ull, 0ull, 0ull };
    for (uint32_t b = threadIdx.x; b < ctas; b += blockDim.x)
    {
      const uint64_t at = (uint64_t)b * nq + q;
      if (at < pcap) fold_add(f, parts[at * 3], parts[at * 3 + 1], parts[at * 3 + 2]);
    }
    for (int o = 16; o > 0; o >>= 1)
    {
      unsigned long long c = __shfl_xor_sync(0xffffffffu, f.c, o);
      unsigned long long lo = __shfl_xor_sync(0xffffffffu, f.lo, o);
      unsigned long long hi = __shfl_xor_sync(0xffffffffu, f.hi, o);
      fold_add(f, c, lo, hi);
    }
    if ((threadIdx.x & 31u) == 0u) s_warp[threadIdx.x >> 5] = f;
    __syncthreads();
    if (threadIdx.x == 0)
    {
      Fold128 t = s_warp[0];
      for (uint32_t w = 1; w < blockDim.x / 32u; w++) fold_add(t, s_warp[w].c, s_warp[w].lo, s_warp[w].hi);
      out[(uint64_t)q * 3] = t.c;
      out[(uint64_t)q * 3 + 1] = t.lo;
      out[(uint64_t)q * 3 + 2] = t.hi;
    }
    __syncthreads();
  }
}

static int launch_batch_fold(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint32_t nq = cql_word(a, 0), ctas = cql_word(a, 2);
  if (nq == 0) return 0;
  if (a.bytes[1] < (uint64_t)nq * 24) return (int)cudaErrorInvalidValue;
  k_batch_fold<<<std::min<uint32_t>(nq, 65535u), SCAN_THREADS, 0, stream>>>(a, nq, ctas);
  CQL_LAUNCH_CHECK();
  return 0;
}

const CqlKernelDesc cql_kernels_scan[] = {
  { "cql_batch_fold", launch_batch_fold },
  { "cql_zone_map", launch_zone_map },
  { "scan_simple", launch_scan_simple },
  { "scan_filter", launch_scan_filter },
  { "cql_bitmap_popc", launch_bitmap_popc },
  { "cql_bitmap_emit", launch_bitmap_emit },
  { nullptr, nullptr },
};
