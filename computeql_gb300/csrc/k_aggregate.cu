// Whole-column and small-range GROUP BY aggregation kernels.
//
//  aggregate_global_native  - contract of src/gpu/vulkan/shaders/aggregate_global_native.comp:1-271
//  aggregate_global_f32     - src/gpu/vulkan/shaders/aggregate_global_f32.comp:1-13, the same kernel with every column F32
//  aggregate_dense_native   - contract of src/gpu/vulkan/shaders/aggregate_dense_native.comp:1-333
//
// GB300 design notes:
//  * FP64 throughput on GB300 is a small fraction of its integer rate, so whole-number columns
//    (U32/I32 and their narrow 1/2-byte codes) are folded in 64-bit integer registers and turned
//    into a double once per CTA. The sums are exact, so the result equals the reference's double
//    fold whenever that fold is exact (every sum below 2^53). F64 columns keep a double sum and
//    fold min/max as order-preserving 64-bit integer keys; F32 columns fold min/max in float.
//  * Loads are 16-byte vectors with the streaming cache hint, four in flight per thread, over a
//    persistent grid of a few CTAs per SM (the reference sizes groups for a 40-CU consumer part).
//  * The dense GROUP BY keeps every group of the key range in shared memory when it fits the
//    227 KB a CTA may use (10k groups fit in one pass: the reference tiles them into 2048-word
//    slices and re-reads the rows per tile), privatised per warp for small group counts.
#include "cql_internal.cuh"
#include <float.h>
#include <algorithm>

#define COLTYPE_U32 1u
#define COLTYPE_F32 3u
#define COLTYPE_F64 4u
#define COLTYPE_I32 7u

#define AGG_THREADS 256

// ---------------------------------------------------------------------------------------------
// aggregate_global_native
//   binding 0..3: the columns; binding 4: partials [workgroup][column][3] doubles (sum, min, max)
//   slot 0: rows, slot 1: column count, slot 2: workgroup count, slot 3+c: type | width<<8 | base<<32

struct GlobalAcc
{
  // whole-number columns
  unsigned long long usum;
  long long ssum;
  unsigned int umin, umax;
  int imin, imax;
  unsigned long long rows;
  // float columns
  double dsum;
  unsigned long long kmin, kmax;  // order keys of f64 values
  float fmin, fmax;
};

__device__ __forceinline__ uint4 ld_stream(const uint4* p) { return __ldcs(p); }

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename T>
__device__ __forceinline__ T warp_min(T v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    T w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    T w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// Block-wide reduction through shared memory: every thread gets the result.
template <typename T, typename Op>
__device__ __forceinline__ T block_reduce(T v, T* sh, Op op)
{
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  T r = sh[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); w++) r = op(r, sh[w]);
  return r;
}

struct OpAddU { __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const { return a + b; } };
struct OpAddS { __device__ long long operator()(long long a, long long b) const { return a + b; } };
struct OpAddD { __device__ double operator()(double a, double b) const { return a + b; } };
struct OpMinU { __device__ unsigned int operator()(unsigned int a, unsigned int b) const { return a < b ? a : b; } };
struct OpMaxU { __device__ unsigned int operator()(unsigned int a, unsigned int b) const { return a > b ? a : b; } };
struct OpMinI { __device__ int operator()(int a, int b) const { return a < b ? a : b; } };
struct OpMaxI { __device__ int operator()(int a, int b) const { return a > b ? a : b; } };
struct OpMinK { __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const { return a < b ? a : b; } };
struct OpMaxK { __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const { return a > b ? a : b; } };
struct OpMinF { __device__ float operator()(float a, float b) const { return fminf(a, b); } };
struct OpMaxF { __device__ float operator()(float a, float b) const { return fmaxf(a, b); } };

// One whole-word U32/I32 column. Sums exact in 64 bits.
template <bool SIGNED>
__device__ void fold_word_column(const uint32_t* col, uint64_t rows, uint64_t t, uint64_t stride, unsigned long long& usum,
                                 long long& ssum, unsigned int& umin, unsigned int& umax, int& imin, int& imax)
{
  const uint4* v = (const uint4*)col;
  uint64_t vec_count = rows / 4;
  uint64_t i = t;
  // four independent 16-byte loads in flight per thread
  for (; i + 3 * stride < vec_count; i += 4 * stride)
  {
    uint4 q[4];
#pragma unroll
    for (int u = 0; u < 4; u++) q[u] = ld_stream(v + i + u * stride);
#pragma unroll
    for (int u = 0; u < 4; u++)
    {
      if (SIGNED)
      {
        int a = (int)q[u].x, b = (int)q[u].y, c = (int)q[u].z, d = (int)q[u].w;
        ssum += (long long)a + (long long)b + (long long)c + (long long)d;
        imin = min(imin, min(min(a, b), min(c, d)));
        imax = max(imax, max(max(a, b), max(c, d)));
      }
      else
      {
        usum += (unsigned long long)q[u].x + q[u].y + (unsigned long long)q[u].z + q[u].w;
        umin = min(umin, min(min(q[u].x, q[u].y), min(q[u].z, q[u].w)));
        umax = max(umax, max(max(q[u].x, q[u].y), max(q[u].z, q[u].w)));
      }
    }
  }
  for (; i < vec_count; i += stride)
  {
    uint4 q = ld_stream(v + i);
    if (SIGNED)
    {
      int a = (int)q.x, b = (int)q.y, c = (int)q.z, d = (int)q.w;
      ssum += (long long)a + (long long)b + (long long)c + (long long)d;
      imin = min(imin, min(min(a, b), min(c, d)));
      imax = max(imax, max(max(a, b), max(c, d)));
    }
    else
    {
      usum += (unsigned long long)q.x + q.y + (unsigned long long)q.z + q.w;
      umin = min(umin, min(min(q.x, q.y), min(q.z, q.w)));
      umax = max(umax, max(max(q.x, q.y), max(q.z, q.w)));
    }
  }
  // rows after the last whole vector, at most 3
  uint64_t tail = vec_count * 4;
  if (t < rows - tail)
  {
    uint32_t w = col[tail + t];
    if (SIGNED)
    {
      ssum += (int)w;
      imin = min(imin, (int)w);
      imax = max(imax, (int)w);
    }
    else
    {
      usum += w;
      umin = min(umin, w);
      umax = max(umax, w);
    }
  }
}

// A narrow column: 1- or 2-byte codes, value = base + code. Codes fold as unsigned whole numbers.
__device__ void fold_narrow_column(const uint32_t* col, uint32_t width, uint64_t rows, uint64_t t, uint64_t stride,
                                   unsigned long long& codes, unsigned int& cmin, unsigned int& cmax, unsigned long long& nrows)
{
  const uint4* v = (const uint4*)col;
  uint32_t per_vec = width == 1 ? 16 : 8;
  uint64_t vec_count = rows / per_vec;
  for (uint64_t i = t; i < vec_count; i += stride)
  {
    uint4 q = ld_stream(v + i);
    uint32_t w[4] = { q.x, q.y, q.z, q.w };
    if (width == 1)
    {
#pragma unroll
      for (int k = 0; k < 4; k++)
      {
        uint32_t x = w[k];
        // byte sums: (x & 0x00ff00ff) + ((x >> 8) & 0x00ff00ff) holds two 10-bit lane sums
        uint32_t pairs = (x & 0x00ff00ffu) + ((x >> 8) & 0x00ff00ffu);
        codes += (pairs & 0xffffu) + (pairs >> 16);
        uint32_t b0 = x & 0xff, b1 = (x >> 8) & 0xff, b2 = (x >> 16) & 0xff, b3 = x >> 24;
        cmin = min(cmin, min(min(b0, b1), min(b2, b3)));
        cmax = max(cmax, max(max(b0, b1), max(b2, b3)));
      }
    }
    else
    {
#pragma unroll
      for (int k = 0; k < 4; k++)
      {
        uint32_t lo = w[k] & 0xffff, hi = w[k] >> 16;
        codes += lo + hi;
        cmin = min(cmin, min(lo, hi));
        cmax = max(cmax, max(lo, hi));
      }
    }
    nrows += per_vec;
  }
  uint64_t tail = vec_count * per_vec;
  if (t < rows - tail)
  {
    uint64_t row = tail + t;
    uint32_t code = width == 1 ? (col[row >> 2] >> ((row & 3) * 8)) & 0xffu : (col[row >> 1] >> ((row & 1) * 16)) & 0xffffu;
    codes += code;
    cmin = min(cmin, code);
    cmax = max(cmax, code);
    nrows += 1;
  }
}

__global__ void __launch_bounds__(AGG_THREADS) k_aggregate_global(CqlLaunch a, uint32_t grid_used)
{
  __shared__ unsigned long long sh_u64[AGG_THREADS / 32];
  __shared__ double sh_f64[AGG_THREADS / 32];
  __shared__ unsigned int sh_u32[AGG_THREADS / 32];
  __shared__ int sh_i32[AGG_THREADS / 32];
  __shared__ float sh_f32[AGG_THREADS / 32];

  uint64_t rows = (uint32_t)a.push[0];
  uint32_t ncols = cql_word(a, 2);
  uint32_t groups = cql_word(a, 4);
  if (ncols > 4) ncols = 4;
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)grid_used * blockDim.x;
  double* partials = (double*)a.buf[4];
  uint64_t partial_cap = a.bytes[4] / sizeof(double);

  for (uint32_t c = 0; c < ncols; c++)
  {
    uint32_t type_word = cql_word(a, 6 + c * 2);
    uint32_t type = type_word & 0xffu;
    uint32_t narrow = (type_word >> 8) & 0xffu;
    uint32_t base = cql_word(a, 7 + c * 2);
    const uint32_t* col = (const uint32_t*)a.buf[c];
    double psum, pmin, pmax;

    if ((narrow == 1 || narrow == 2) && (type == COLTYPE_U32 || type == COLTYPE_I32))
    {
      unsigned long long codes = 0, n = 0;
      unsigned int cmin = 0xffffffffu, cmax = 0;
      fold_narrow_column(col, narrow, rows, t, stride, codes, cmin, cmax, n);
      codes = block_reduce(codes, sh_u64, OpAddU());
      n = block_reduce(n, sh_u64, OpAddU());
      cmin = block_reduce(cmin, sh_u32, OpMinU());
      cmax = block_reduce(cmax, sh_u32, OpMaxU());
      if (n > 0)
      {
        long long b = type == COLTYPE_I32 ? (long long)(int)base : (long long)base;
        psum = (double)((long long)codes + b * (long long)n);
        pmin = (double)(b + (long long)cmin);
        pmax = (double)(b + (long long)cmax);
      }
      else
      {
        psum = 0.0;
        pmin = DBL_MAX;
        pmax = -DBL_MAX;
      }
    }
    else if (type == COLTYPE_U32 || type == COLTYPE_I32)
    {
      unsigned long long usum = 0;
      long long ssum = 0;
      unsigned int umin = 0xffffffffu, umax = 0;
      int imin = 0x7fffffff, imax = (int)0x80000000;
      if (type == COLTYPE_I32) fold_word_column<true>(col, rows, t, stride, usum, ssum, umin, umax, imin, imax);
      else fold_word_column<false>(col, rows, t, stride, usum, ssum, umin, umax, imin, imax);
      // a CTA that saw no row leaves the reference's +-biggest double
      uint64_t vecs = rows / 4;
      int seen = (t < vecs) || (t < rows - vecs * 4);
      int any = block_reduce(seen, sh_i32, OpMaxI());
      if (type == COLTYPE_I32)
      {
        ssum = block_reduce(ssum, (long long*)sh_u64, OpAddS());
        imin = block_reduce(imin, sh_i32, OpMinI());
        imax = block_reduce(imax, sh_i32, OpMaxI());
        psum = (double)ssum;
        pmin = any ? (double)imin : DBL_MAX;
        pmax = any ? (double)imax : -DBL_MAX;
      }
      else
      {
        usum = block_reduce(usum, sh_u64, OpAddU());
        umin = block_reduce(umin, sh_u32, OpMinU());
        umax = block_reduce(umax, sh_u32, OpMaxU());
        psum = (double)usum;
        pmin = any ? (double)umin : DBL_MAX;
        pmax = any ? (double)umax : -DBL_MAX;
      }
    }
    else if (type == COLTYPE_F64)
    {
      const uint4* v = (const uint4*)col;
      uint64_t vec_count = rows / 2;
      double dsum = 0.0;
      unsigned long long kmin = ~0ull, kmax = 0ull;
      uint64_t i = t;
      for (; i + 3 * stride < vec_count; i += 4 * stride)
      {
        uint4 q[4];
#pragma unroll
        for (int u = 0; u < 4; u++) q[u] = ld_stream(v + i + u * stride);
#pragma unroll
        for (int u = 0; u < 4; u++)
        {
          double x0 = __hiloint2double((int)q[u].y, (int)q[u].x);
          double x1 = __hiloint2double((int)q[u].w, (int)q[u].z);
          dsum += x0 + x1;
          unsigned long long k0 = cql_f64_order_key(x0), k1 = cql_f64_order_key(x1);
          kmin = min(kmin, min(k0, k1));
          kmax = max(kmax, max(k0, k1));
        }
      }
      for (; i < vec_count; i += stride)
      {
        uint4 q = ld_stream(v + i);
        double x0 = __hiloint2double((int)q.y, (int)q.x);
        double x1 = __hiloint2double((int)q.w, (int)q.z);
        dsum += x0 + x1;
        unsigned long long k0 = cql_f64_order_key(x0), k1 = cql_f64_order_key(x1);
        kmin = min(kmin, min(k0, k1));
        kmax = max(kmax, max(k0, k1));
      }
      if (t == 0 && (rows & 1))
      {
        double x = ((const double*)col)[rows - 1];
        dsum += x;
        unsigned long long k = cql_f64_order_key(x);
        kmin = min(kmin, k);
        kmax = max(kmax, k);
      }
      dsum = block_reduce(dsum, sh_f64, OpAddD());
      kmin = block_reduce(kmin, sh_u64, OpMinK());
      kmax = block_reduce(kmax, sh_u64, OpMaxK());
      psum = dsum;
      pmin = kmin == ~0ull ? DBL_MAX : cql_f64_from_order_key(kmin);
      pmax = kmax == 0ull ? -DBL_MAX : cql_f64_from_order_key(kmax);
    }
    else
    {
      // F32 widened to double for the sum, min/max compared as floats (widening keeps the order)
      const uint4* v = (const uint4*)col;
      uint64_t vec_count = rows / 4;
      double dsum = 0.0;
      float fmn = FLT_MAX, fmx = -FLT_MAX;
      int seen = 0;
      for (uint64_t i = t; i < vec_count; i += stride)
      {
        uint4 q = ld_stream(v + i);
        float x0 = __uint_as_float(q.x), x1 = __uint_as_float(q.y), x2 = __uint_as_float(q.z), x3 = __uint_as_float(q.w);
        dsum += ((double)x0 + (double)x1) + ((double)x2 + (double)x3);
        fmn = fminf(fmn, fminf(fminf(x0, x1), fminf(x2, x3)));
        fmx = fmaxf(fmx, fmaxf(fmaxf(x0, x1), fmaxf(x2, x3)));
        seen = 1;
      }
      uint64_t tail = vec_count * 4;
      if (t < rows - tail)
      {
        float x = __uint_as_float(col[tail + t]);
        dsum += (double)x;
        fmn = fminf(fmn, x);
        fmx = fmaxf(fmx, x);
        seen = 1;
      }
      dsum = block_reduce(dsum, sh_f64, OpAddD());
      fmn = block_reduce(fmn, sh_f32, OpMinF());
      fmx = block_reduce(fmx, sh_f32, OpMaxF());
      int any = block_reduce(seen, sh_i32, OpMaxI());
      psum = dsum;
      pmin = any ? (double)fmn : DBL_MAX;
      pmax = any ? (double)fmx : -DBL_MAX;
    }

    if (threadIdx.x == 0)
    {
      uint64_t at = ((uint64_t)blockIdx.x * ncols + c) * 3;
      if (at + 2 < partial_cap)
      {
        partials[at + 0] = psum;
        partials[at + 1] = pmin;
        partials[at + 2] = pmax;
      }
    }
    __syncthreads();
  }

  // workgroups the reference would have launched but this grid did not: neutral partials
  for (uint64_t w = grid_used + blockIdx.x; w < groups; w += grid_used)
  {
    for (uint32_t i = threadIdx.x; i < ncols * 3; i += blockDim.x)
    {
      uint64_t at = w * ncols * 3 + i;
      if (at < partial_cap)
      {
        uint32_t part = i % 3;
        partials[at] = part == 0 ? 0.0 : (part == 1 ? DBL_MAX : -DBL_MAX);
      }
    }
  }
}

static int launch_aggregate_global(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint32_t groups = cql_word(a, 4);
  uint64_t rows = (uint32_t)a.push[0];
  if (groups == 0) return 0;
  // enough CTAs to keep ~64 KB of loads in flight per SM, never more than the reference's workgroups
  uint64_t need = (rows / 4 + AGG_THREADS - 1) / AGG_THREADS;
  uint32_t grid = cql_stream_grid(need ? need : 1, 4);
  if (grid > groups) grid = groups;
  k_aggregate_global<<<grid, AGG_THREADS, 0, stream>>>(a, grid);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// aggregate_dense_native
//   binding 0: key column; 1..4: argument columns; 5: info [group][2] (word 1 = row count);
//   6: sums [group][expr] as (lo, hi) words; 7: mins [group][expr]; 8: maxs [group][expr]
//   word 0 rows; word 1 widths (key bits 0-3, arg a bits 4+4a); word 2 exprs; word 3 base of arg 0;
//   word 4 funcs (4 bits each); word 5 base of arg 1; word 6 arg index per expr; word 7 signed bits
//   (bit 31: narrow sums); word 8 groups; word 9 base of arg 2; word 10 min key (and key base when
//   narrow); word 11 base of arg 3; words 12-14 the reference's tiling; word 15 chunk's first row

#define FUNC_COUNT 0u
#define FUNC_SUM   1u
#define FUNC_AVG   2u
#define FUNC_MIN   3u
#define FUNC_MAX   4u

struct DenseDecode
{
  const uint32_t* col[5];  // key, arg0..3
  uint32_t log2w[5], bits[5], mask[5], base[5];
  bool seq[5];
  uint32_t chunk_start;
};

__device__ __forceinline__ uint32_t dense_read(const DenseDecode& d, int c, uint64_t row)
{
  if (d.seq[c]) return d.base[c] + d.chunk_start + (uint32_t)row;
  uint32_t l = d.log2w[c];
  uint32_t w = d.col[c][row >> l];
  uint32_t sh = (uint32_t)((row & ((1u << l) - 1u)) * d.bits[c]) & 31u;
  return d.base[c] + ((w >> sh) & d.mask[c]);
}

struct DenseLayout
{
  uint32_t groups;        // groups in this pass
  uint32_t exprs;
  uint32_t nsum, nmm;     // expressions needing a sum slot / a min+max slot
  uint32_t copies;        // privatised copies of the table
  uint32_t copy_words;    // 32-bit words per copy (sums are 2 words, 8-byte aligned)
  uint32_t sum_off, mm_off;
  uint32_t sum_slot[8], mm_slot[8];
};

// words per group of one copy: count, then 2 words per summed expr, then 2 words per min/max expr
__host__ __device__ inline uint32_t dense_group_words(uint32_t nsum, uint32_t nmm) { return 1 + 2 * nsum + 2 * nmm; }

template <bool WIDE_VEC>
__global__ void __launch_bounds__(1024) k_aggregate_dense(CqlLaunch a, DenseLayout L, uint32_t group_base, uint64_t rows)
{
  extern __shared__ __align__(16) uint32_t smem[];
  DenseDecode d;
  uint32_t widths = cql_word(a, 1);
  uint32_t arg_base[4] = { cql_word(a, 3), cql_word(a, 5), cql_word(a, 9), cql_word(a, 11) };
  for (int c = 0; c < 5; c++)
  {
    uint32_t w = (widths >> (4 * c)) & 0xfu;
    d.col[c] = (const uint32_t*)a.buf[c];
    d.log2w[c] = w == 1 ? 2 : (w == 2 ? 1 : 0);
    d.bits[c] = w == 1 ? 8 : (w == 2 ? 16 : 32);
    d.mask[c] = w == 1 ? 0xffu : (w == 2 ? 0xffffu : 0xffffffffu);
    if (c == 0) d.base[c] = (w == 1 || w == 2) ? cql_word(a, 10) : 0u;
    else d.base[c] = (w == 1 || w == 2 || w == 3) ? arg_base[c - 1] : 0u;
    d.seq[c] = c > 0 && w == 3;
  }
  d.chunk_start = cql_word(a, 15);
  uint32_t func_codes = cql_word(a, 4);
  uint32_t arg_index = cql_word(a, 6);
  uint32_t arg_signed = cql_word(a, 7);
  int min_key = (int)cql_word(a, 10);

  // per copy: [count | sums (8-byte aligned) | min,max] for each group
  uint32_t G = L.groups;
  uint32_t total = L.copies * L.copy_words;
  for (uint32_t i = threadIdx.x; i < total; i += blockDim.x)
  {
    uint32_t in_copy = i % L.copy_words;
    uint32_t v = 0;
    if (in_copy >= L.mm_off)
    {
      uint32_t k = in_copy - L.mm_off;
      v = (k & 1u) ? 0x80000000u : 0x7fffffffu;  // min then max per (group, expr)
    }
    smem[i] = v;
  }
  __syncthreads();

  uint32_t copy = (threadIdx.x >> 5) % L.copies;
  uint32_t* cnt = smem + copy * L.copy_words;
  unsigned long long* sums = (unsigned long long*)(smem + copy * L.copy_words + L.sum_off);
  int* mm = (int*)(smem + copy * L.copy_words + L.mm_off);

  auto count_row = [&](uint64_t row, uint32_t key) {
    int id = (int)key - min_key - (int)group_base;
    if (id < 0 || (uint32_t)id >= G) return;
    atomicAdd(&cnt[id], 1u);
    for (uint32_t e = 0; e < L.exprs; e++)
    {
      uint32_t f = (func_codes >> (e * 4)) & 0xfu;
      if (f == FUNC_COUNT) continue;
      uint32_t ai = (arg_index >> (e * 4)) & 0x3u;  // at most 4 argument columns are bound
      uint32_t word = dense_read(d, 1 + (int)ai, row);
      if (f == FUNC_SUM || f == FUNC_AVG)
      {
        bool is_signed = ((arg_signed >> ai) & 1u) != 0u;
        unsigned long long add = is_signed ? (unsigned long long)(long long)(int)word : (unsigned long long)word;
        atomicAdd(&sums[(uint32_t)id * L.nsum + L.sum_slot[e]], add);
      }
      else if (f == FUNC_MIN)
        atomicMin(&mm[((uint32_t)id * L.nmm + L.mm_slot[e]) * 2], (int)word);
      else if (f == FUNC_MAX)
        atomicMax(&mm[((uint32_t)id * L.nmm + L.mm_slot[e]) * 2 + 1], (int)word);
    }
  };

  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (WIDE_VEC)
  {
    // whole-word key: four keys per 16-byte load, two vectors in flight
    const uint4* kv = (const uint4*)d.col[0];
    uint64_t vec_count = rows / 4;
    uint64_t i = t;
    for (; i + stride < vec_count; i += 2 * stride)
    {
      uint4 q0 = __ldcs(kv + i);
      uint4 q1 = __ldcs(kv + i + stride);
      uint64_t r0 = i * 4, r1 = (i + stride) * 4;
      count_row(r0 + 0, q0.x);
      count_row(r0 + 1, q0.y);
      count_row(r0 + 2, q0.z);
      count_row(r0 + 3, q0.w);
      count_row(r1 + 0, q1.x);
      count_row(r1 + 1, q1.y);
      count_row(r1 + 2, q1.z);
      count_row(r1 + 3, q1.w);
    }
    for (; i < vec_count; i += stride)
    {
      uint4 q = __ldcs(kv + i);
      uint64_t r = i * 4;
      count_row(r + 0, q.x);
      count_row(r + 1, q.y);
      count_row(r + 2, q.z);
      count_row(r + 3, q.w);
    }
    uint64_t tail = vec_count * 4;
    if (t < rows - tail) count_row(tail + t, d.col[0][tail + t]);
  }
  else
  {
    for (uint64_t row = t; row < rows; row += stride) count_row(row, dense_read(d, 0, row));
  }
  __syncthreads();

  // fold the copies and merge into the global arrays, skipping groups this CTA never saw
  uint32_t* info = (uint32_t*)a.buf[5];
  unsigned long long* gsum = (unsigned long long*)a.buf[6];
  int* gmin = (int*)a.buf[7];
  int* gmax = (int*)a.buf[8];
  uint64_t info_cap = a.bytes[5] / 4, sum_cap = a.bytes[6] / 8, mm_cap_min = a.bytes[7] / 4, mm_cap_max = a.bytes[8] / 4;
  for (uint32_t g = threadIdx.x; g < G; g += blockDim.x)
  {
    uint32_t count = 0;
    for (uint32_t c = 0; c < L.copies; c++) count += smem[c * L.copy_words + g];
    if (count == 0) continue;
    uint64_t gg = (uint64_t)group_base + g;
    if (gg * 2 + 1 < info_cap) atomicAdd(&info[gg * 2 + 1], count);
    for (uint32_t e = 0; e < L.exprs; e++)
    {
      uint32_t f = (func_codes >> (e * 4)) & 0xfu;
      uint64_t index = gg * L.exprs + e;
      if (f == FUNC_SUM || f == FUNC_AVG)
      {
        unsigned long long s = 0;
        for (uint32_t c = 0; c < L.copies; c++)
          s += ((unsigned long long*)(smem + c * L.copy_words + L.sum_off))[g * L.nsum + L.sum_slot[e]];
        if (index < sum_cap) atomicAdd(&gsum[index], s);
      }
      else if (f == FUNC_MIN || f == FUNC_MAX)
      {
        int best = f == FUNC_MIN ? 0x7fffffff : (int)0x80000000;
        for (uint32_t c = 0; c < L.copies; c++)
        {
          int v = ((int*)(smem + c * L.copy_words + L.mm_off))[(g * L.nmm + L.mm_slot[e]) * 2 + (f == FUNC_MAX ? 1 : 0)];
          best = f == FUNC_MIN ? min(best, v) : max(best, v);
        }
        if (f == FUNC_MIN && index < mm_cap_min) atomicMin(&gmin[index], best);
        if (f == FUNC_MAX && index < mm_cap_max) atomicMax(&gmax[index], best);
      }
    }
  }
}


// Fast path for whole-word keys and argument columns (the full-width u32/i32 case): per-expression
// metadata unrolled into registers, key and argument vectors loaded together (16 bytes each), 32-bit
// shared atomics with a carry into the high word as aggregate_dense_native.comp:184-200 does, one
// private table per warp when the groups are few. KEYARG: the one argument column is the key column
// itself (GROUP BY amount ... SUM(amount)), read once.
// DEPTH: key vectors (and vectors of every argument column) in flight per thread. 2 where several CTAs share an
// SM; 4 for the one-CTA-an-SM tables (1024 threads, a table of thousands of groups), whose warps alone must keep
// enough loads in flight.
template <int NE, int NA, bool KEYARG = false, int DEPTH = 2>
__global__ void __launch_bounds__(1024) k_aggregate_dense_wide(CqlLaunch a, uint32_t G, uint32_t group_base, uint64_t rows,
                                                               uint32_t copies, uint32_t copy_words, uint32_t nsum)
{
  extern __shared__ __align__(16) uint32_t smem[];
  uint32_t func_codes = cql_word(a, 4);
  uint32_t arg_index = cql_word(a, 6);
  uint32_t arg_signed = cql_word(a, 7);
  int min_key = (int)cql_word(a, 10);
  uint32_t f[NE], ai[NE], sg[NE], slot[NE];
  uint32_t ns = 0, nm = 0;
#pragma unroll
  for (int e = 0; e < NE; e++)
  {
    f[e] = (func_codes >> (4 * e)) & 0xfu;
    ai[e] = (arg_index >> (4 * e)) & 0x3u;
    sg[e] = (arg_signed >> ai[e]) & 1u;
    slot[e] = 0;
    if (f[e] == FUNC_SUM || f[e] == FUNC_AVG) slot[e] = ns++;
    else if (f[e] == FUNC_MIN || f[e] == FUNC_MAX) slot[e] = nm++;
  }
  uint32_t mm_off = G + 2 * G * nsum;
  for (uint32_t i = threadIdx.x; i < copies * copy_words; i += blockDim.x)
  {
    uint32_t in_copy = i % copy_words;
    uint32_t v = 0;
    if (in_copy >= mm_off)
    {
      uint32_t k = in_copy - mm_off;          // [slot][min G | max G]
      v = ((k / G) & 1u) ? 0x80000000u : 0x7fffffffu;
    }
    smem[i] = v;
  }
  __syncthreads();
  uint32_t copy = (threadIdx.x >> 5) % copies;
  uint32_t* cnt = smem + copy * copy_words;
  uint32_t* sums = cnt + G;
  int* mm = (int*)(cnt + mm_off);

  auto row = [&](uint32_t key, const uint32_t* v) {
    uint32_t id = (uint32_t)((int)key - min_key - (int)group_base);
    if (id >= G) return;
    atomicAdd(&cnt[id], 1u);
    // the argument is the key: its SUM is key x count and its MIN and MAX the key, set at the fold
    if constexpr (!KEYARG)
    {
#pragma unroll
      for (int e = 0; e < NE; e++)
      {
        if (f[e] == FUNC_COUNT) continue;
        uint32_t x = v[0];
#pragma unroll
        for (int c = 1; c < NA; c++)
          if (ai[e] == (uint32_t)c) x = v[c];
        if (f[e] == FUNC_SUM || f[e] == FUNC_AVG)
        {
          uint32_t* lo = sums + slot[e] * 2 * G;
          uint32_t old = atomicAdd(&lo[id], x);
          uint32_t hi_add = ((sg[e] && (int)x < 0) ? 0xffffffffu : 0u) + ((old + x < old) ? 1u : 0u);
          if (hi_add) atomicAdd(&lo[G + id], hi_add);
        }
        else if (f[e] == FUNC_MIN)
          atomicMin(&mm[slot[e] * 2 * G + id], (int)x);
        else if (f[e] == FUNC_MAX)
          atomicMax(&mm[slot[e] * 2 * G + G + id], (int)x);
      }
    }
  };

  const uint4* kv = (const uint4*)a.buf[0];
  uint64_t vec_count = rows / 4;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int NC = NA > 0 ? NA : 1;
  uint64_t i = t;
  // DEPTH key vectors and DEPTH vectors of every argument column in flight per thread
  for (; i + (uint64_t)(DEPTH - 1) * stride < vec_count; i += DEPTH * stride)
  {
    uint4 kk[DEPTH], qq[DEPTH][NC];
#pragma unroll
    for (int dd = 0; dd < DEPTH; dd++)
    {
      kk[dd] = __ldcs(kv + i + dd * stride);
#pragma unroll
      for (int c = 0; c < NC; c++)
      {
        if (KEYARG) qq[dd][c] = kk[dd];
        else if (c < NA) qq[dd][c] = __ldcs((const uint4*)a.buf[1 + c] + i + dd * stride);
        else qq[dd][c] = make_uint4(0, 0, 0, 0);
      }
    }
#pragma unroll
    for (int dd = 0; dd < DEPTH; dd++)
    {
      uint32_t v[NC];
#pragma unroll
      for (int c = 0; c < NC; c++) v[c] = qq[dd][c].x;
      row(kk[dd].x, v);
#pragma unroll
      for (int c = 0; c < NC; c++) v[c] = qq[dd][c].y;
      row(kk[dd].y, v);
#pragma unroll
      for (int c = 0; c < NC; c++) v[c] = qq[dd][c].z;
      row(kk[dd].z, v);
#pragma unroll
      for (int c = 0; c < NC; c++) v[c] = qq[dd][c].w;
      row(kk[dd].w, v);
    }
  }
  for (; i < vec_count; i += stride)
  {
    uint4 k0 = __ldcs(kv + i);
    uint4 q0[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) q0[c] = c < NA ? (KEYARG ? k0 : __ldcs((const uint4*)a.buf[1 + c] + i)) : make_uint4(0, 0, 0, 0);
    uint32_t v[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) v[c] = q0[c].x;
    row(k0.x, v);
#pragma unroll
    for (int c = 0; c < NC; c++) v[c] = q0[c].y;
    row(k0.y, v);
#pragma unroll
    for (int c = 0; c < NC; c++) v[c] = q0[c].z;
    row(k0.z, v);
#pragma unroll
    for (int c = 0; c < NC; c++) v[c] = q0[c].w;
    row(k0.w, v);
  }
  uint64_t tail = vec_count * 4;
  if (t < rows - tail)
  {
    uint64_t r = tail + t;
    uint32_t v[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) v[c] = c < NA ? ((const uint32_t*)a.buf[1 + c])[r] : 0u;
    row(((const uint32_t*)a.buf[0])[r], v);
  }
  __syncthreads();

  uint32_t* info = (uint32_t*)a.buf[5];
  unsigned long long* gsum = (unsigned long long*)a.buf[6];
  int* gmin = (int*)a.buf[7];
  int* gmax = (int*)a.buf[8];
  uint64_t info_cap = a.bytes[5] / 4, sum_cap = a.bytes[6] / 8, min_cap = a.bytes[7] / 4, max_cap = a.bytes[8] / 4;
  for (uint32_t g = threadIdx.x; g < G; g += blockDim.x)
  {
    uint32_t count = 0;
    for (uint32_t c = 0; c < copies; c++) count += smem[c * copy_words + g];
    if (count == 0) continue;
    uint64_t gg = (uint64_t)group_base + g;
    if (gg * 2 + 1 < info_cap) atomicAdd(&info[gg * 2 + 1], count);
#pragma unroll
    for (int e = 0; e < NE; e++)
    {
      uint64_t index = gg * NE + e;
      if (KEYARG && f[e] != FUNC_COUNT)
      {
        uint32_t key = (uint32_t)(min_key + (int)gg);
        unsigned long long value = sg[e] ? (unsigned long long)(long long)(int)key : (unsigned long long)key;
        if ((f[e] == FUNC_SUM || f[e] == FUNC_AVG) && index < sum_cap) atomicAdd(&gsum[index], value * count);
        if (f[e] == FUNC_MIN && index < min_cap) atomicMin(&gmin[index], (int)key);
        if (f[e] == FUNC_MAX && index < max_cap) atomicMax(&gmax[index], (int)key);
        continue;
      }
      if (f[e] == FUNC_SUM || f[e] == FUNC_AVG)
      {
        unsigned long long total = 0;
        for (uint32_t c = 0; c < copies; c++)
        {
          const uint32_t* lo = smem + c * copy_words + G + slot[e] * 2 * G;
          total += ((unsigned long long)lo[G + g] << 32) | lo[g];
        }
        if (index < sum_cap) atomicAdd(&gsum[index], total);
      }
      else if (f[e] == FUNC_MIN || f[e] == FUNC_MAX)
      {
        int best = f[e] == FUNC_MIN ? 0x7fffffff : (int)0x80000000;
        for (uint32_t c = 0; c < copies; c++)
        {
          const int* m = (const int*)(smem + c * copy_words + mm_off) + slot[e] * 2 * G;
          best = f[e] == FUNC_MIN ? min(best, m[g]) : max(best, m[G + g]);
        }
        if (f[e] == FUNC_MIN && index < min_cap) atomicMin(&gmin[index], best);
        if (f[e] == FUNC_MAX && index < max_cap) atomicMax(&gmax[index], best);
      }
    }
  }
}

typedef void (*DenseWideFn)(CqlLaunch, uint32_t, uint32_t, uint64_t, uint32_t, uint32_t, uint32_t);
// four vectors in flight for the one-CTA-an-SM tables of the common shapes (up to 4 aggregates over up to 2
// argument columns, and the key-is-the-argument form with up to 2 aggregates)
#define DW4_ROW(NE) { k_aggregate_dense_wide<NE, 0, false, 4>, k_aggregate_dense_wide<NE, 1, false, 4>, k_aggregate_dense_wide<NE, 2, false, 4> }
static const DenseWideFn k_dense_wide_deep[4][3] = { DW4_ROW(1), DW4_ROW(2), DW4_ROW(3), DW4_ROW(4) };
static const DenseWideFn k_dense_keyarg_deep[2] = { k_aggregate_dense_wide<1, 1, true, 4>, k_aggregate_dense_wide<2, 1, true, 4> };
#define DW_ROW(NE) { k_aggregate_dense_wide<NE, 0>, k_aggregate_dense_wide<NE, 1>, k_aggregate_dense_wide<NE, 2>, k_aggregate_dense_wide<NE, 4> }
static const DenseWideFn k_dense_wide_table[8][4] = { DW_ROW(1), DW_ROW(2), DW_ROW(3), DW_ROW(4), DW_ROW(5), DW_ROW(6), DW_ROW(7), DW_ROW(8) };
static const DenseWideFn k_dense_keyarg_table[8] = { k_aggregate_dense_wide<1, 1, true>, k_aggregate_dense_wide<2, 1, true>,
                                                     k_aggregate_dense_wide<3, 1, true>, k_aggregate_dense_wide<4, 1, true>,
                                                     k_aggregate_dense_wide<5, 1, true>, k_aggregate_dense_wide<6, 1, true>,
                                                     k_aggregate_dense_wide<7, 1, true>, k_aggregate_dense_wide<8, 1, true> };
#undef DW_ROW

// Whole-word key and arguments: one pass per tile of groups that fits shared memory.
static int launch_dense_wide(const CqlLaunch& a, uint64_t rows, uint32_t exprs, uint32_t groups, uint32_t nsum, uint32_t nmm, cudaStream_t stream)
{
  uint32_t per_group = 1 + 2 * nsum + 2 * nmm;
  uint32_t budget_words = (uint32_t)(std::min(g_cql_max_smem_optin, 200 * 1024) / 4);
  uint32_t tile = std::min<uint32_t>(groups, budget_words / per_group);
  if (tile == 0) return (int)cudaErrorInvalidValue;
  // distinct argument columns are bound at 1..n in order (qe_dense_stream_core, query_exec.c:7863-7867)
  uint32_t funcs = cql_word(a, 4), arg_index = cql_word(a, 6), na = 0;
  for (uint32_t e = 0; e < exprs; e++)
  {
    uint32_t f = (funcs >> (4 * e)) & 0xfu;
    if (f != FUNC_COUNT) na = std::max(na, ((arg_index >> (4 * e)) & 0x3u) + 1);
  }
  bool keyarg = na == 1 && a.buf[1] == a.buf[0];
  for (uint32_t base = 0; base < groups; base += tile)
  {
    uint32_t G = std::min(tile, groups - base);
    uint32_t copy_words = (G * per_group + 3) & ~3u;
    uint32_t threads = copy_words * 4 > 48 * 1024 ? 1024 : 512;
    DenseWideFn fn = keyarg ? k_dense_keyarg_table[exprs - 1] : k_dense_wide_table[exprs - 1][na <= 2 ? na : 3];
    if (threads == 1024 && keyarg && exprs <= 2) fn = k_dense_keyarg_deep[exprs - 1];
    else if (threads == 1024 && !keyarg && exprs <= 4 && na <= 2) fn = k_dense_wide_deep[exprs - 1][na];
    uint32_t copies = 1;
    while (copies < threads / 32 && (uint64_t)copy_words * 4 * copies * 2 <= 32 * 1024) copies *= 2;
    size_t smem = (size_t)copy_words * 4 * copies;
    if (smem > 48 * 1024) cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (int)threads, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
    uint64_t need = (rows / 4 + threads - 1) / threads;
    uint32_t grid = cql_stream_grid(need ? need : 1, per_sm);
    fn<<<grid, threads, smem, stream>>>(a, G, base, rows, copies, copy_words, nsum);
    CQL_LAUNCH_CHECK();
  }
  return 0;
}

static int launch_aggregate_dense(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = cql_word(a, 0);
  uint32_t widths = cql_word(a, 1);
  uint32_t exprs = cql_word(a, 2);
  uint32_t funcs = cql_word(a, 4);
  uint32_t groups = cql_word(a, 8);
  if (exprs > 8 || groups == 0 || rows == 0) return 0;

  DenseLayout L;
  L.exprs = exprs;
  L.nsum = 0;
  L.nmm = 0;
  for (uint32_t e = 0; e < 8; e++)
  {
    L.sum_slot[e] = 0;
    L.mm_slot[e] = 0;
  }
  for (uint32_t e = 0; e < exprs; e++)
  {
    uint32_t f = (funcs >> (e * 4)) & 0xfu;
    if (f == FUNC_SUM || f == FUNC_AVG) L.sum_slot[e] = L.nsum++;
    if (f == FUNC_MIN || f == FUNC_MAX) L.mm_slot[e] = L.nmm++;
  }
  // whole-word key and arguments take the fast path
  bool all_wide = true;
  for (uint32_t c = 0; c < 5; c++)
  {
    uint32_t w = (widths >> (4 * c)) & 0xfu;
    if (!(w == 0 || w == 4)) all_wide = false;
  }
  if (all_wide) return launch_dense_wide(a, rows, exprs, groups, L.nsum, L.nmm, stream);

  uint32_t per_group_words = dense_group_words(L.nsum, L.nmm);
  uint32_t budget_words = (uint32_t)(std::min(g_cql_max_smem_optin, 200 * 1024) / 4);
  uint32_t tile = groups;
  if ((uint64_t)tile * per_group_words + 4 > budget_words) tile = (budget_words - 4) / per_group_words;
  if (tile == 0) return (int)cudaErrorInvalidValue;

  bool wide = (widths & 0xfu) == 0 || (widths & 0xfu) == 4;
  for (uint32_t base = 0; base < groups; base += tile)
  {
    uint32_t G = std::min(tile, groups - base);
    L.groups = G;
    // words of one copy: counts (padded to even), sums (2 words each), min/max pairs
    uint32_t cnt_words = (G + 1) & ~1u;
    L.sum_off = cnt_words;
    L.mm_off = L.sum_off + 2 * G * L.nsum;
    L.copy_words = L.mm_off + 2 * G * L.nmm;
    L.copy_words = (L.copy_words + 3) & ~3u;
    // few groups: one copy per warp so 32 lanes of 16 warps do not serialise on the same words
    uint32_t threads = L.copy_words * 4 > 64 * 1024 ? 1024 : 512;
    uint32_t warps = threads / 32;
    uint32_t copies = 1;
    while (copies < warps && (uint64_t)L.copy_words * 4 * copies * 2 <= 48 * 1024 && G <= 4096) copies *= 2;
    L.copies = copies;
    size_t smem = (size_t)L.copy_words * 4 * copies;
    int per_sm = 1;
    if (smem <= 24 * 1024) per_sm = threads == 512 ? 4 : 2;
    else if (smem <= 48 * 1024) per_sm = threads == 512 ? 3 : 2;
    else if (smem <= 100 * 1024) per_sm = 2;
    if (threads == 1024 && per_sm > 2) per_sm = 2;
    if (smem > 48 * 1024)
    {
      if (wide) cudaFuncSetAttribute(k_aggregate_dense<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      else cudaFuncSetAttribute(k_aggregate_dense<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    uint64_t need = (rows / (wide ? 4 : 1) + threads - 1) / threads;
    uint32_t grid = cql_stream_grid(need ? need : 1, per_sm);
    if (wide) k_aggregate_dense<true><<<grid, threads, smem, stream>>>(a, L, base, rows);
    else k_aggregate_dense<false><<<grid, threads, smem, stream>>>(a, L, base, rows);
    CQL_LAUNCH_CHECK();
  }
  return 0;
}

// aggregate_global_f32.comp:1-13 has the same bindings and slots 0-2 but no type words: every column is F32
static int launch_aggregate_global_f32(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  CqlLaunch b = a;
  for (int c = 0; c < 4; c++) b.push[3 + c] = COLTYPE_F32;
  return launch_aggregate_global(b, gws, lws, stream);
}

const CqlKernelDesc cql_kernels_aggregate[] = {
  { "aggregate_global_native", launch_aggregate_global },
  { "aggregate_global_f32", launch_aggregate_global_f32 },
  { "aggregate_dense_native", launch_aggregate_dense },
  { nullptr, nullptr },
};
