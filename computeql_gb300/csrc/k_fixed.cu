// Fixed-point decimals: GROUP BY over a small-range whole-number key with f64/f32 arguments that are
// decimals of at most 6 places, aggregated exactly as scaled integers.
//
//  cql_fixed_scale        the scale qe_values_fixed_point finds for a column (src/query_exec/query_exec.c:3893-3983)
//  cql_key_range          the smallest and largest key, and whether every key is a whole number
//  aggregate_dense_f64    src/gpu/vulkan/shaders/aggregate_dense_f64.comp:1-190 (binding and push layout kept)
//  aggregate_dense_f32    src/gpu/vulkan/shaders/aggregate_dense_f32.comp (the same with float arguments)
//  cql_dense_fixed        the same reduce over typed device columns (u32/i32/f64 key, f64/f32 arguments,
//                         an optional row selection) so nothing is gathered to f64 on the host first
//
// The reference decides "v has scale s" with FP64 arithmetic (whole = (S64)(v*10^s +- 0.5), then
// whole / 10^s == v) and scales each argument as floor(v*10^s + 0.5). FP64 is a small fraction of
// GB300's issue rate, so both are done here in integer arithmetic on the double's bits, exactly:
// with |v| = m * 2^-sh, W = floor(m*10^s / 2^sh + 1/2) is the nearest integer to |v|*10^s, and
// whole / 10^s == v holds exactly when W / 10^s rounds to v, i.e. when W*2^sh - m*10^s lies inside
// v's rounding interval (half an ulp either side, a quarter below a power of two, ties to the even
// mantissa). For |v| < 2^31 and s <= 6 the reference's rounded product and the exact one give the
// same W whenever the test can pass, and the property is monotone in s (whole at s => whole at s+1),
// so the smallest passing scale of each value, maximised over the values, is the scale the
// reference's running search reaches in any order.
#include "cql_internal.cuh"
#include <algorithm>
#include <climits>

#define FIX_THREADS 256
#define FUNC_COUNT 0u
#define FUNC_SUM 1u
#define FUNC_AVG 2u
#define FUNC_MIN 3u
#define FUNC_MAX 4u
#define TYPE_U32 1u
#define TYPE_F32 3u
#define TYPE_F64 4u
#define TYPE_I32 7u

#include "cql_fixed.cuh"

// ---------------------------------------------------------------------------------------------
// cql_fixed_scale: binding 0 values, 1 result (u32 max scale, u32 failed, u64 max |v| f64 bits; zeroed
// by the caller), 2 selection (u32 rows), 3 per-value scale (i8, -1 = none) when word 6 is 1;
// word 0 n, word 2 type (F64 4 / F32 3), word 4 1 = the n values are the selection's rows

template <bool F32>
__device__ __forceinline__ FixVal fix_load(const void* values, uint64_t r)
{
  if (F32) return fix_decode_f32(((const uint32_t*)values)[r]);
  return fix_decode_f64(((const unsigned long long*)values)[r]);
}

template <bool F32>
__global__ void __launch_bounds__(FIX_THREADS) k_fixed_scale(CqlLaunch a, uint64_t n)
{
  const void* values = a.buf[0];
  uint32_t* result = (uint32_t*)a.buf[1];
  const uint32_t* sel = (const uint32_t*)a.buf[2];
  int8_t* per_value = (int8_t*)a.buf[3];
  bool selected = cql_word(a, 4) != 0, each = cql_word(a, 6) != 0;
  int scale = 0;
  bool failed = false;
  unsigned long long largest = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    FixVal f = fix_load<F32>(values, selected ? sel[i] : i);
    int s = each ? 0 : scale;
    unsigned long long w;
    bool ok = !f.big;
    if (ok)
    {
      while (!fix_whole(f, s, &w))
        if (++s > FIXED_MAX_SCALE) break;
      ok = s <= FIXED_MAX_SCALE;
    }
    if (each) per_value[i] = ok ? (int8_t)s : (int8_t)-1;
    if (!ok)
    {
      failed = true;
      if (!each) break;
      continue;
    }
    scale = max(scale, s);
    largest = max(largest, f.mag_bits);
  }
  // reduced over the warp, then the CTA, then one atomic of each kind a CTA (atomics a warp would all meet on
  // the same three words)
  __shared__ uint32_t s_failed, s_scale;
  __shared__ unsigned long long s_largest;
  if (threadIdx.x == 0)
  {
    s_failed = 0;
    s_scale = 0;
    s_largest = 0;
  }
  __syncthreads();
  uint32_t any_failed = __any_sync(0xffffffffu, failed);
  int wscale = __reduce_max_sync(0xffffffffu, (unsigned)scale);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) largest = max(largest, __shfl_xor_sync(0xffffffffu, largest, o));
  if ((threadIdx.x & 31u) == 0)
  {
    if (any_failed) s_failed = 1u;
    if (wscale) atomicMax(&s_scale, (unsigned)wscale);
    if (largest) atomicMax(&s_largest, largest);
  }
  __syncthreads();
  if (threadIdx.x == 0)
  {
    if (s_failed) atomicOr(&result[1], 1u);
    if (s_scale) atomicMax(&result[0], s_scale);
    if (s_largest) atomicMax((unsigned long long*)(result + 2), s_largest);
  }
}

static int launch_fixed_scale(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t n = cql_word(a, 0);
  uint32_t type = cql_word(a, 2);
  if (n == 0) return 0;
  bool f32 = type == TYPE_F32;
  if ((type != TYPE_F32 && type != TYPE_F64) || a.bytes[1] < 16) return (int)cudaErrorInvalidValue;
  bool selected = cql_word(a, 4) != 0;
  if (selected ? a.bytes[2] < n * 4 : a.bytes[0] < n * (f32 ? 4 : 8)) return (int)cudaErrorInvalidValue;
  if (cql_word(a, 6) && a.bytes[3] < n) return (int)cudaErrorInvalidValue;
  uint32_t grid = cql_stream_grid((n + FIX_THREADS - 1) / FIX_THREADS, 8);
  if (f32) k_fixed_scale<true><<<grid, FIX_THREADS, 0, stream>>>(a, n);
  else k_fixed_scale<false><<<grid, FIX_THREADS, 0, stream>>>(a, n);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// cql_key_range: binding 0 keys, 1 result (i64 min, i64 max, u32 not-whole-or-out-of-range flag; the
// caller fills min with INT64_MAX and max with INT64_MIN), 2 selection; word 0 n, word 2 type
// (U32/I32/F64), word 4 1 = selection. An f64 key must be a whole number inside the i32 range.

__device__ __forceinline__ bool key_value(uint32_t type, const void* keys, uint64_t r, long long* out)
{
  if (type == TYPE_U32)
  {
    *out = ((const uint32_t*)keys)[r];
    return true;
  }
  if (type == TYPE_I32)
  {
    *out = ((const int*)keys)[r];
    return true;
  }
  FixVal f = fix_decode_f64(((const unsigned long long*)keys)[r]);
  if (f.big) return false;
  // whole: the bits below 2^0 are zero
  long long v;
  if (f.sh <= 0) v = (long long)(f.m << (-f.sh));
  else if (f.sh >= 64) { if (f.m) return false; v = 0; }
  else
  {
    if (f.m & ((1ull << f.sh) - 1ull)) return false;
    v = (long long)(f.m >> f.sh);
  }
  *out = f.neg ? -v : v;
  return true;
}

__global__ void __launch_bounds__(FIX_THREADS) k_key_range(CqlLaunch a, uint64_t n)
{
  const void* keys = a.buf[0];
  long long* result = (long long*)a.buf[1];
  const uint32_t* sel = (const uint32_t*)a.buf[2];
  uint32_t type = cql_word(a, 2);
  bool selected = cql_word(a, 4) != 0;
  long long lo = LLONG_MAX, hi = LLONG_MIN;
  bool bad = false;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    long long v;
    if (!key_value(type, keys, selected ? sel[i] : i, &v))
    {
      bad = true;
      continue;
    }
    lo = min(lo, v);
    hi = max(hi, v);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  bool any_bad = __any_sync(0xffffffffu, bad);
  // over the CTA first, then one atomic of each kind a CTA
  __shared__ long long s_lo, s_hi;
  __shared__ uint32_t s_bad;
  if (threadIdx.x == 0)
  {
    s_lo = LLONG_MAX;
    s_hi = LLONG_MIN;
    s_bad = 0;
  }
  __syncthreads();
  if ((threadIdx.x & 31u) == 0)
  {
    atomicMin(&s_lo, lo);
    atomicMax(&s_hi, hi);
    if (any_bad) s_bad = 1u;
  }
  __syncthreads();
  if (threadIdx.x == 0)
  {
    atomicMin(&result[0], s_lo);
    atomicMax(&result[1], s_hi);
    if (s_bad) atomicOr((unsigned*)&result[2], 1u);
  }
}

static int launch_key_range(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t n = cql_word(a, 0);
  uint32_t type = cql_word(a, 2);
  if (n == 0) return 0;
  if ((type != TYPE_U32 && type != TYPE_I32 && type != TYPE_F64) || a.bytes[1] < 24) return (int)cudaErrorInvalidValue;
  bool selected = cql_word(a, 4) != 0;
  if (selected ? a.bytes[2] < n * 4 : a.bytes[0] < n * (type == TYPE_F64 ? 8 : 4)) return (int)cudaErrorInvalidValue;
  k_key_range<<<cql_stream_grid((n + FIX_THREADS - 1) / FIX_THREADS, 8), FIX_THREADS, 0, stream>>>(a, n);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// The dense fixed-point reduce. Bindings (aggregate_dense_f64.comp:22-36): 0 keys, 1 info per group
// (complement of its smallest row, row count), 2 sums per group and expression (low, high word),
// 3 min per group and expression (i32), 4 max (i32), 5..12 the arguments of expressions 0..7;
// words 0 rows, 2 expressions, 4 function codes (4 bits each), 6 scales (4 bits each), 8 groups,
// 10 smallest key (i32). cql_dense_fixed adds word 12 the key type (U32/I32/F64), word 13 a bit per
// expression whose argument is F32 (else F64), word 14 1 = the rows are binding 13's selection.
//
// Shared memory per copy: per group [smallest row, count, (low, high) x E] then [min, max] x E.
// Few groups get a copy per warp (lanes of many warps would serialise on one group's words).

struct DenseFixedArgs
{
  uint32_t exprs, funcs, scales, groups, arg_f32;
  int min_key;
  uint32_t acc_stride, copy_words, copies;
  uint64_t row_limit;   // rows every bound column holds (a selected row at or past it is skipped)
};

// One row into the shared table. owner[e] is the first expression reading the same argument at the
// same scale, whose scaled value expression e reuses (SUM, MIN and MAX of one column decode it once).
__device__ __forceinline__ void fixed_row(const CqlLaunch& a, const DenseFixedArgs& p, uint32_t* acc, int* mm, uint32_t key_type,
                                          const void* keys, uint64_t r, uint32_t row_number, const uint32_t* owner)
{
  long long kv;
  if (!key_value(key_type, keys, r, &kv)) return;   // an f64 key is int(keys[row]) of a whole number
  long long id = kv - (long long)p.min_key;
  if (id < 0 || id >= (long long)p.groups) return;
  uint32_t* g = acc + (uint32_t)id * p.acc_stride;
  int* gm = mm + (uint32_t)id * 2 * p.exprs;
  atomicMin(&g[0], row_number);
  atomicAdd(&g[1], 1u);
  int qv[8];
#pragma unroll
  for (uint32_t e = 0; e < 8; e++)
  {
    qv[e] = 0;
    if (e >= p.exprs) continue;
    uint32_t f = (p.funcs >> (4 * e)) & 0xfu;
    if (f == FUNC_COUNT) continue;
    int q;
    if (owner[e] == e)
    {
      int s = (int)min((p.scales >> (4 * e)) & 0xfu, (uint32_t)FIXED_MAX_SCALE);
      const void* arg = a.buf[5 + e];
      FixVal fv = ((p.arg_f32 >> e) & 1u) ? fix_decode_f32(((const uint32_t*)arg)[r]) : fix_decode_f64(((const unsigned long long*)arg)[r]);
      q = fix_scaled(fv, s);
    }
    else
    {
      q = 0;
#pragma unroll
      for (uint32_t o = 0; o < e; o++)
        if (owner[e] == o) q = qv[o];
    }
    qv[e] = q;
    if (f == FUNC_SUM || f == FUNC_AVG)
    {
      uint32_t low = (uint32_t)q;
      uint32_t before = atomicAdd(&g[2 + 2 * e], low);
      uint32_t high_add = (q < 0 ? 0xffffffffu : 0u) + (before + low < before ? 1u : 0u);
      if (high_add) atomicAdd(&g[3 + 2 * e], high_add);
    }
    else if (f == FUNC_MIN)
      atomicMin(&gm[2 * e], q);
    else if (f == FUNC_MAX)
      atomicMax(&gm[2 * e + 1], q);
  }
}

__global__ void __launch_bounds__(FIX_THREADS) k_dense_fixed(CqlLaunch a, DenseFixedArgs p, uint64_t rows, uint32_t key_type, int selected)
{
  extern __shared__ __align__(16) uint32_t smem[];
  uint32_t acc_words = p.groups * p.acc_stride;
  for (uint32_t i = threadIdx.x; i < p.copies * p.copy_words; i += blockDim.x)
  {
    uint32_t in_copy = i % p.copy_words;
    uint32_t v;
    if (in_copy < acc_words) v = (in_copy % p.acc_stride) == 0 ? 0xffffffffu : 0u;
    else v = ((in_copy - acc_words) & 1u) ? 0x80000000u : 0x7fffffffu;
    smem[i] = v;
  }
  __syncthreads();
  uint32_t copy = (threadIdx.x >> 5) % p.copies;
  uint32_t* acc = smem + copy * p.copy_words;
  int* mm = (int*)(acc + acc_words);
  const void* keys = a.buf[0];
  const uint32_t* sel = (const uint32_t*)a.buf[13];
  uint32_t owner[8];
#pragma unroll
  for (uint32_t e = 0; e < 8; e++)
  {
    owner[e] = e;
    for (uint32_t o = 0; o < e && e < p.exprs; o++)
    {
      uint32_t fo = (p.funcs >> (4 * o)) & 0xfu;
      if (owner[e] == e && fo != FUNC_COUNT && a.buf[5 + o] == a.buf[5 + e] && ((p.arg_f32 >> o) & 1u) == ((p.arg_f32 >> e) & 1u) &&
          ((p.scales >> (4 * o)) & 0xfu) == ((p.scales >> (4 * e)) & 0xfu))
        owner[e] = o;
    }
  }
  // four consecutive rows per thread and step: their loads are in flight together
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x * 4;
  for (uint64_t i0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4; i0 < rows; i0 += stride)
  {
#pragma unroll
    for (uint32_t j = 0; j < 4; j++)
    {
      uint64_t i = i0 + j;
      if (i >= rows) break;
      uint64_t r = selected ? sel[i] : i;
      if (r < p.row_limit) fixed_row(a, p, acc, mm, key_type, keys, r, (uint32_t)r, owner);
    }
  }
  __syncthreads();
  uint32_t* info = (uint32_t*)a.buf[1];
  unsigned long long* sums = (unsigned long long*)a.buf[2];
  int* gmin = (int*)a.buf[3];
  int* gmax = (int*)a.buf[4];
  for (uint32_t g = threadIdx.x; g < p.groups; g += blockDim.x)
  {
    uint32_t count = 0, first = 0xffffffffu;
    for (uint32_t c = 0; c < p.copies; c++)
    {
      const uint32_t* ga = smem + c * p.copy_words + g * p.acc_stride;
      count += ga[1];
      first = min(first, ga[0]);
    }
    if (count == 0) continue;
    // the smallest row is kept as its complement so that a zeroed buffer and atomicMax pick it
    atomicMax(&info[g * 2], ~first);
    atomicAdd(&info[g * 2 + 1], count);
    for (uint32_t e = 0; e < p.exprs; e++)
    {
      uint32_t f = (p.funcs >> (4 * e)) & 0xfu;
      uint64_t index = (uint64_t)g * p.exprs + e;
      if (f == FUNC_SUM || f == FUNC_AVG)
      {
        unsigned long long total = 0;
        for (uint32_t c = 0; c < p.copies; c++)
        {
          const uint32_t* ga = smem + c * p.copy_words + g * p.acc_stride;
          total += ((unsigned long long)ga[3 + 2 * e] << 32) | ga[2 + 2 * e];
        }
        atomicAdd(&sums[index], total);
      }
      else if (f == FUNC_MIN || f == FUNC_MAX)
      {
        int best = f == FUNC_MIN ? 0x7fffffff : (int)0x80000000;
        for (uint32_t c = 0; c < p.copies; c++)
        {
          const int* gm = (const int*)(smem + c * p.copy_words + acc_words) + g * 2 * p.exprs;
          best = f == FUNC_MIN ? min(best, gm[2 * e]) : max(best, gm[2 * e + 1]);
        }
        if (f == FUNC_MIN) atomicMin(&gmin[index], best);
        else atomicMax(&gmax[index], best);
      }
    }
  }
}

static int launch_dense_fixed_common(const CqlLaunch& a, uint32_t key_type, uint32_t arg_f32, int selected, cudaStream_t stream)
{
  uint64_t rows = cql_word(a, 0);
  DenseFixedArgs p;
  p.exprs = cql_word(a, 2);
  p.funcs = cql_word(a, 4);
  p.scales = cql_word(a, 6);
  p.groups = cql_word(a, 8);
  p.min_key = (int)cql_word(a, 10);
  p.arg_f32 = arg_f32;
  if (rows == 0 || p.groups == 0) return 0;
  if (p.exprs == 0 || p.exprs > 8) return (int)cudaErrorInvalidValue;
  uint64_t key_bytes = key_type == TYPE_F64 ? 8 : 4;
  if (selected ? a.bytes[13] < rows * 4 : a.bytes[0] < rows * key_bytes) return (int)cudaErrorInvalidValue;
  uint64_t entries = (uint64_t)p.groups * p.exprs;
  if (a.bytes[1] < (uint64_t)p.groups * 8 || a.bytes[2] < entries * 8 || a.bytes[3] < entries * 4 || a.bytes[4] < entries * 4)
    return (int)cudaErrorInvalidValue;
  p.row_limit = a.bytes[0] / key_bytes;
  for (uint32_t e = 0; e < p.exprs; e++)
  {
    uint32_t f = (p.funcs >> (4 * e)) & 0xfu;
    if (f > FUNC_MAX) return (int)cudaErrorInvalidValue;
    if (f == FUNC_COUNT) continue;
    uint64_t arg_rows = a.bytes[5 + e] / (((arg_f32 >> e) & 1u) ? 4 : 8);
    if (!selected && arg_rows < rows) return (int)cudaErrorInvalidValue;
    p.row_limit = std::min(p.row_limit, arg_rows);
  }
  p.acc_stride = 2 + 2 * p.exprs;
  uint64_t words = (uint64_t)p.groups * (p.acc_stride + 2 * p.exprs);
  uint64_t budget = (uint64_t)std::min(g_cql_max_smem_optin, 200 * 1024) / 4;
  if (words > budget) return (int)cudaErrorInvalidValue;
  p.copy_words = (uint32_t)((words + 3) & ~3ull);
  p.copies = 1;
  while (p.copies < FIX_THREADS / 32 && (uint64_t)p.copy_words * 4 * p.copies * 2 <= 32 * 1024) p.copies *= 2;
  size_t smem = (size_t)p.copy_words * 4 * p.copies;
  if (smem > 48 * 1024) cudaFuncSetAttribute((const void*)k_dense_fixed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dense_fixed, FIX_THREADS, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
  uint32_t grid = cql_stream_grid((rows + FIX_THREADS - 1) / FIX_THREADS, per_sm);
  k_dense_fixed<<<grid, FIX_THREADS, smem, stream>>>(a, p, rows, key_type, selected);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_dense_f64(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  return launch_dense_fixed_common(a, TYPE_F64, 0u, 0, stream);
}

static int launch_dense_f32(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  return launch_dense_fixed_common(a, TYPE_F64, 0xffu, 0, stream);
}

static int launch_dense_typed(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint32_t key_type = cql_word(a, 12);
  if (key_type != TYPE_U32 && key_type != TYPE_I32 && key_type != TYPE_F64) return (int)cudaErrorInvalidValue;
  return launch_dense_fixed_common(a, key_type, cql_word(a, 13) & 0xffu, cql_word(a, 14) != 0, stream);
}

const CqlKernelDesc cql_kernels_fixed[] = {
  { "cql_fixed_scale", launch_fixed_scale },
  { "cql_key_range", launch_key_range },
  { "aggregate_dense_f64", launch_dense_f64 },
  { "aggregate_dense_f32", launch_dense_f32 },
  { "cql_dense_fixed", launch_dense_typed },
  { nullptr, nullptr },
};
