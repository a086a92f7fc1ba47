// Hash joins.
//
//  hash_join_build_count  src/gpu/vulkan/shaders/hash_join_build_count.comp:1-81  bucket histogram of the build keys
//  prefix_sum / _sum2     src/gpu/vulkan/shaders/prefix_sum.comp:1-103            exclusive scan in three modes, seeds the cursor
//  hash_join_probe        src/gpu/vulkan/shaders/hash_join_probe.comp:1-137       probe rows emit (probe, build) pairs, LEFT JOIN unmatched
//  join_pack_key          src/gpu/vulkan/shaders/join_pack_key.comp:1-52          two whole-number keys folded into one f64 key
//  join_probe_native      src/gpu/vulkan/shaders/join_probe_native.comp:1-238     fact-side probe fused with per-dim-row aggregates
//
// Keys are f64 values (or raw strings) hashed from their bit patterns exactly as the reference does, so a
// build row lands in the same bucket. GB300 design: persistent grid-stride launches; the fused probe keeps
// eight keys and their Bloom words in flight per thread and bounds every open-addressing walk by the
// table size (the reference's walk assumes an empty slot exists).
#include "cql_internal.cuh"
#include <algorithm>

#define JOIN_THREADS 256
#define BUILD_NULL 0xffffffffu

__device__ __forceinline__ uint32_t jhash_u32(uint32_t x)
{
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ uint32_t num_hash(const uint32_t* data, uint64_t row)
{
  uint32_t lo = data[row * 2], hi = data[row * 2 + 1];
  return jhash_u32(lo ^ jhash_u32(hi));
}

// ---------------------------------------------------------------------------------------------
// hash_join_build_count: binding 0 build keys, 1 build offsets, 2 bucket counts, 3 bucket per row;
// words 0 rows, 2 buckets, 4 string key

__global__ void __launch_bounds__(JOIN_THREADS) k_join_build_count(CqlLaunch a, uint64_t rows)
{
  const uint32_t* data = (const uint32_t*)a.buf[0];
  const uint32_t* off = (const uint32_t*)a.buf[1];
  uint32_t* counts = (uint32_t*)a.buf[2];
  uint32_t* row_bucket = (uint32_t*)a.buf[3];
  uint32_t buckets = cql_word(a, 2);
  bool is_str = cql_word(a, 4) != 0;
  if (!buckets) return;
  for (uint64_t row = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; row < rows; row += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t h;
    if (is_str)
    {
      uint32_t s = off[row * 2], e = off[(row + 1) * 2];
      h = 2166136261u;
      const unsigned char* b = (const unsigned char*)data;
      for (uint32_t i = s; i < e; i++) h = (h ^ b[i]) * 16777619u;
    }
    else h = num_hash(data, row);
    uint32_t bucket = h % buckets;
    row_bucket[row] = bucket;
    atomicAdd(&counts[bucket], 1u);
  }
}

static int launch_join_build_count(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = cql_word(a, 0);
  if (rows == 0) return 0;
  k_join_build_count<<<cql_stream_grid((rows + JOIN_THREADS - 1) / JOIN_THREADS, 8), JOIN_THREADS, 0, stream>>>(a, rows);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// prefix_sum: binding 0 counts, 1 offsets (n + 1), 2 cursor, 3 block totals; word 0 n, word 2 mode

__device__ uint32_t join_block_scan(uint32_t v, uint32_t* sh, uint32_t* total)
{
  uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl += y;
  }
  if (lane == 31) sh[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    uint32_t run = 0;
    for (int w = 0; w < JOIN_THREADS / 32; w++)
    {
      uint32_t t = sh[w];
      sh[w] = run;
      run += t;
    }
    sh[JOIN_THREADS / 32] = run;
  }
  __syncthreads();
  uint32_t ex = sh[warp] + incl - v;
  *total = sh[JOIN_THREADS / 32];
  __syncthreads();
  return ex;
}

__global__ void __launch_bounds__(JOIN_THREADS) k_prefix_sum(CqlLaunch a, uint32_t mode, uint32_t n)
{
  __shared__ uint32_t sh[JOIN_THREADS / 32 + 1];
  const uint32_t* counts = (const uint32_t*)a.buf[0];
  uint32_t* offsets = (uint32_t*)a.buf[1];
  uint32_t* cursor = (uint32_t*)a.buf[2];
  uint32_t* block_sums = (uint32_t*)a.buf[3];
  uint32_t blocks = (n + 255) / 256;
  uint32_t total;
  if (mode == 0)
  {
    for (uint32_t b = blockIdx.x; b < blocks; b += gridDim.x)
    {
      uint32_t index = b * 256 + threadIdx.x;
      uint32_t v = index < n ? counts[index] : 0u;
      uint32_t ex = join_block_scan(v, sh, &total);
      if (index < n) offsets[index] = ex;
      if (threadIdx.x == 0) block_sums[b] = total;
    }
  }
  else if (mode == 1)
  {
    if (blockIdx.x != 0) return;
    uint32_t chunk = (blocks + 255) / 256;
    uint32_t start = min(threadIdx.x * chunk, blocks), end = min(start + chunk, blocks);
    uint32_t sum = 0;
    for (uint32_t i = start; i < end; i++) sum += block_sums[i];
    uint32_t running = join_block_scan(sum, sh, &total);
    for (uint32_t i = start; i < end; i++)
    {
      uint32_t t = block_sums[i];
      block_sums[i] = running;
      running += t;
    }
    if (threadIdx.x == 0) offsets[n] = total;
  }
  else
  {
    for (uint64_t index = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; index < n; index += (uint64_t)gridDim.x * blockDim.x)
    {
      uint32_t t = offsets[index] + block_sums[index / 256];
      offsets[index] = t;
      cursor[index] = t;
    }
  }
}

static int launch_prefix_sum(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint32_t n = cql_word(a, 0), mode = cql_word(a, 2);
  uint32_t blocks = (n + 255) / 256;
  if (mode == 1) k_prefix_sum<<<1, JOIN_THREADS, 0, stream>>>(a, mode, n);
  else k_prefix_sum<<<cql_stream_grid(blocks ? blocks : 1, 8), JOIN_THREADS, 0, stream>>>(a, mode, n);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// hash_join_probe: binding 0/1 build keys + offsets, 2 bucket offsets (buckets + 1), 3 bucket rows,
// 4/5 probe keys + offsets, 6 pairs (probe, 0, build, 0) x capacity, 7 pair count;
// words 0 probe rows, 2 buckets, 4 left join, 6 string key, 8 capacity

__device__ bool str_equal(const uint32_t* bd, const uint32_t* bo, uint64_t brow, const uint32_t* pd, const uint32_t* po, uint64_t prow)
{
  uint32_t bs = bo[brow * 2], be = bo[(brow + 1) * 2], ps = po[prow * 2], pe = po[(prow + 1) * 2];
  if (be - bs != pe - ps) return false;
  const unsigned char* b = (const unsigned char*)bd;
  const unsigned char* p = (const unsigned char*)pd;
  for (uint32_t i = 0; i < be - bs; i++)
    if (b[bs + i] != p[ps + i]) return false;
  return true;
}

__global__ void __launch_bounds__(JOIN_THREADS) k_join_probe(CqlLaunch a, uint64_t probe_rows)
{
  const uint32_t* bd = (const uint32_t*)a.buf[0];
  const uint32_t* bo = (const uint32_t*)a.buf[1];
  const uint32_t* bucket_off = (const uint32_t*)a.buf[2];
  const uint32_t* bucket_rows = (const uint32_t*)a.buf[3];
  const uint32_t* pd = (const uint32_t*)a.buf[4];
  const uint32_t* po = (const uint32_t*)a.buf[5];
  uint32_t* pairs = (uint32_t*)a.buf[6];
  uint32_t* count = (uint32_t*)a.buf[7];
  uint32_t buckets = cql_word(a, 2), capacity = cql_word(a, 8);
  bool left = cql_word(a, 4) != 0, is_str = cql_word(a, 6) != 0;
  uint64_t cap_words = a.bytes[6] / 16;
  if (cap_words < capacity) capacity = (uint32_t)cap_words;
  if (!buckets) return;
  uint32_t lane = threadIdx.x & 31u;
  // whole warps take every iteration: a warp counts its lanes' pairs, takes their places with one
  // atomic on the pair count (one per pair serialised on that counter), then writes them
  for (uint64_t row = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; row - lane < probe_rows; row += (uint64_t)gridDim.x * blockDim.x)
  {
    bool valid = row < probe_rows;
    uint32_t start = 0, end = 0;
    double pv = 0.0;
    if (valid)
    {
      uint32_t h;
      if (is_str)
      {
        uint32_t s = po[row * 2], e = po[(row + 1) * 2];
        h = 2166136261u;
        const unsigned char* b = (const unsigned char*)pd;
        for (uint32_t i = s; i < e; i++) h = (h ^ b[i]) * 16777619u;
      }
      else
      {
        h = num_hash(pd, row);
        pv = __hiloint2double((int)pd[row * 2 + 1], (int)pd[row * 2]);
      }
      uint32_t bucket = h % buckets;
      start = bucket_off[bucket];
      end = bucket_off[bucket + 1];
    }
    uint32_t matches = 0;
    for (uint32_t m = start; m < end; m++)
    {
      uint32_t brow = bucket_rows[m];
      if (is_str ? str_equal(bd, bo, brow, pd, po, row) : (__hiloint2double((int)bd[brow * 2 + 1], (int)bd[brow * 2]) == pv)) matches++;
    }
    uint32_t out = matches ? matches : (valid && left ? 1u : 0u);
    uint32_t incl = out;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t base = 0;
    if (lane == 0 && total) base = atomicAdd(count, total);
    base = __shfl_sync(0xffffffffu, base, 0);
    uint64_t pos = (uint64_t)base + incl - out;
    if (matches)
    {
      for (uint32_t m = start; m < end; m++)
      {
        uint32_t brow = bucket_rows[m];
        if (is_str ? str_equal(bd, bo, brow, pd, po, row) : (__hiloint2double((int)bd[brow * 2 + 1], (int)bd[brow * 2]) == pv))
        {
          if (pos < capacity) *(uint4*)(pairs + pos * 4) = make_uint4((uint32_t)row, 0u, brow, 0u);
          pos++;
        }
      }
    }
    else if (out && pos < capacity) *(uint4*)(pairs + pos * 4) = make_uint4((uint32_t)row, 0u, BUILD_NULL, BUILD_NULL);
  }
}

static int launch_join_probe(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = cql_word(a, 0);
  if (rows == 0) return 0;
  k_join_probe<<<cql_stream_grid((rows + JOIN_THREADS - 1) / JOIN_THREADS, 8), JOIN_THREADS, 0, stream>>>(a, rows);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// join_pack_key: binding 0/1 the two f64 keys, 2 the packed f64 key; word 0 count, slots 1-4 the
// f64 min of each key and their spans (from the build side)

__global__ void __launch_bounds__(JOIN_THREADS) k_join_pack_key(CqlLaunch a, uint64_t count)
{
  const double* first = (const double*)a.buf[0];
  const double* second = (const double*)a.buf[1];
  double* dest = (double*)a.buf[2];
  double min_first = __longlong_as_double((long long)a.push[1]), min_second = __longlong_as_double((long long)a.push[2]);
  double span_first = __longlong_as_double((long long)a.push[3]), span_second = __longlong_as_double((long long)a.push[4]);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x)
  {
    double x = first[i] - min_first, y = second[i] - min_second;
    double key = -1.0;
    if (x >= 0.0 && x < span_first && y >= 0.0 && y < span_second) key = x * span_second + y;
    dest[i] = key;
  }
}

static int launch_join_pack_key(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t count = cql_word(a, 0);
  if (count == 0) return 0;
  k_join_pack_key<<<cql_stream_grid((count + JOIN_THREADS - 1) / JOIN_THREADS, 8), JOIN_THREADS, 0, stream>>>(a, count);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// join_probe_native: binding 0 fact key, 1..4 arguments, 5 table keys, 6 table row + 1 (0 empty),
// 7 counts per dim row, 8 sums (lo, hi), 9 mins, 10 maxs, 11 Bloom words.
// word 0 rows, 1 widths (key bits 0-3, arg a bits 4+4a), 2 exprs, 3 base of arg 0, 4 funcs, 5 base of
// arg 1, 6 arg index per expr, 7 signed bits, 8 table mask, 9 base of arg 2, 10 key base, 11 base of
// arg 3, 12 log2 table size, 13 log2 Bloom words

#define JFUNC_COUNT 0u
#define JFUNC_SUM 1u
#define JFUNC_AVG 2u
#define JFUNC_MIN 3u
#define JFUNC_MAX 4u

struct JoinDecode
{
  const uint32_t* col[5];
  uint32_t log2w[5], bits[5], mask[5], base[5];
};

// PLAIN: every column bound at its full 32-bit width (no narrow codes to unpack)
template <bool PLAIN>
__device__ __forceinline__ uint32_t join_read_t(const JoinDecode& d, int c, uint64_t row)
{
  if (PLAIN) return d.col[c][row];
  uint32_t l = d.log2w[c];
  uint32_t w = d.col[c][row >> l];
  uint32_t sh = (uint32_t)((row & ((1u << l) - 1u)) * d.bits[c]) & 31u;
  return d.base[c] + ((w >> sh) & d.mask[c]);
}

__device__ __forceinline__ uint32_t join_read(const JoinDecode& d, int c, uint64_t row)
{
  uint32_t l = d.log2w[c];
  uint32_t w = d.col[c][row >> l];
  uint32_t sh = (uint32_t)((row & ((1u << l) - 1u)) * d.bits[c]) & 31u;
  return d.base[c] + ((w >> sh) & d.mask[c]);
}

__global__ void __launch_bounds__(JOIN_THREADS, 3) k_join_probe_native(CqlLaunch a, uint64_t rows)
{
  JoinDecode d;
  uint32_t widths = cql_word(a, 1);
  uint32_t arg_base[4] = { cql_word(a, 3), cql_word(a, 5), cql_word(a, 9), cql_word(a, 11) };
#pragma unroll
  for (int c = 0; c < 5; c++)
  {
    uint32_t w = (widths >> (4 * c)) & 0xfu;
    d.col[c] = (const uint32_t*)a.buf[c];
    d.log2w[c] = w == 1 ? 2 : (w == 2 ? 1 : 0);
    d.bits[c] = w == 1 ? 8 : (w == 2 ? 16 : 32);
    d.mask[c] = w == 1 ? 0xffu : (w == 2 ? 0xffffu : 0xffffffffu);
    d.base[c] = (w == 1 || w == 2) ? (c == 0 ? cql_word(a, 10) : arg_base[c - 1]) : 0u;
  }
  const uint32_t* tkeys = (const uint32_t*)a.buf[5];
  const uint32_t* trows = (const uint32_t*)a.buf[6];
  uint32_t* counts = (uint32_t*)a.buf[7];
  unsigned long long* sums = (unsigned long long*)a.buf[8];
  int* mins = (int*)a.buf[9];
  int* maxs = (int*)a.buf[10];
  const uint32_t* bloom = (const uint32_t*)a.buf[11];
  uint32_t exprs = min(cql_word(a, 2), 8u), funcs = cql_word(a, 4), arg_index = cql_word(a, 6), arg_signed = cql_word(a, 7);
  uint32_t mask = cql_word(a, 8), log2_size = cql_word(a, 12), bloom_log2 = cql_word(a, 13);
  uint32_t used_args = 0;   // the argument columns some aggregate reads
  for (uint32_t e = 0; e < exprs; e++)
    if (((funcs >> (e * 4)) & 0xfu) != JFUNC_COUNT) used_args |= 1u << ((arg_index >> (e * 4)) & 0x3u);
  uint32_t table_size = mask + 1;
  uint64_t count_cap = a.bytes[7] / 4;
  const uint32_t UNROLL = 8;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; base < rows; base += stride * UNROLL)
  {
    uint32_t key[UNROLL];
    bool maybe[UNROLL];
#pragma unroll
    for (uint32_t u = 0; u < UNROLL; u++)
    {
      uint64_t at = base + u * stride;
      key[u] = at < rows ? join_read(d, 0, at) : 0u;
    }
#pragma unroll
    for (uint32_t u = 0; u < UNROLL; u++)
    {
      uint64_t at = base + u * stride;
      uint32_t h = key[u] * 0x9E3779B1u, h2 = key[u] * 0x85EBCA6Bu;
      uint32_t bits = (1u << ((h2 >> 27) & 31u)) | (1u << ((h2 >> 22) & 31u));
      maybe[u] = at < rows && (bloom[h >> (32u - bloom_log2)] & bits) == bits;
    }
    // every candidate's first table slot and argument words are loaded before any is used: the loads of
    // the eight rows are in flight together instead of one probe's latency after another's
    uint32_t slot0[UNROLL], key0[UNROLL], row0[UNROLL], argv[UNROLL][4];
#pragma unroll
    for (uint32_t u = 0; u < UNROLL; u++)
    {
      slot0[u] = (key[u] * 0x9E3779B1u) >> (32u - log2_size);
      key0[u] = maybe[u] ? tkeys[slot0[u]] : 0u;
      row0[u] = maybe[u] ? trows[slot0[u]] : 0u;
#pragma unroll
      for (uint32_t c = 0; c < 4; c++) argv[u][c] = (maybe[u] && ((used_args >> c) & 1u)) ? join_read(d, 1 + (int)c, base + u * stride) : 0u;
    }
#pragma unroll
    for (uint32_t u = 0; u < UNROLL; u++)
    {
      if (!maybe[u]) continue;
      uint32_t slot = slot0[u];
      uint32_t found = 0;
      if (row0[u] != 0u && key0[u] == key[u]) found = row0[u];
      else if (row0[u] != 0u)
      {
        slot = (slot + 1u) & mask;
        for (uint32_t probe = 1; probe < table_size; probe++)
        {
          uint32_t r1 = trows[slot];
          if (r1 == 0u) break;
          if (tkeys[slot] == key[u])
          {
            found = r1;
            break;
          }
          slot = (slot + 1u) & mask;
        }
      }
      if (!found) continue;
      uint32_t dim_row = found - 1u;
      if (dim_row >= count_cap) continue;
      atomicAdd(&counts[dim_row], 1u);
      for (uint32_t e = 0; e < exprs; e++)
      {
        uint32_t f = (funcs >> (e * 4)) & 0xfu;
        if (f == JFUNC_COUNT) continue;
        uint32_t ai = (arg_index >> (e * 4)) & 0x3u;
        uint32_t w = ai == 0u ? argv[u][0] : ai == 1u ? argv[u][1] : ai == 2u ? argv[u][2] : argv[u][3];
        uint64_t index = (uint64_t)dim_row * exprs + e;
        if (f == JFUNC_SUM || f == JFUNC_AVG)
        {
          bool sg = ((arg_signed >> ai) & 1u) != 0;
          atomicAdd(&sums[index], sg ? (unsigned long long)(long long)(int)w : (unsigned long long)w);
        }
        else if (f == JFUNC_MIN) atomicMin(&mins[index], (int)w);
        else if (f == JFUNC_MAX) atomicMax(&maxs[index], (int)w);
      }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// join_probe_native over a small build side: the per-dim-row totals are kept per table slot in shared
// memory and flushed to the dim-row arrays once per CTA, instead of a global atomic per matched row. With
// TSMEM the table (keys and rows) and the Bloom words are staged into shared memory too, once per CTA, by
// bulk copies (cp.async.bulk, completion counted on an mbarrier); without it (a table too large to stage
// beside the totals) they are read from global memory, where they stay in L2. The shared arrays hold only
// what the aggregates need: a count per slot, a 64-bit sum (two 32-bit halves) per SUM/AVG, an extremum
// per MIN or MAX. Binding 12 is an error word (bit 0: the staging did not complete within a second; the CTA
// then waits, again bounded, for its copies and returns without probing). Taken when the error word is
// bound and the shared arrays fit; the same results as k_join_probe_native.

#define JOIN_SMEM_THREADS 512
#define JOIN_SMEM_TWO_CTAS (100u * 1024u)    // two CTAs an SM up to this size, one beyond it
#define JOIN_SMEM_MAX_BYTES (200u * 1024u)
#define JOIN_WAIT_NS 1000000000ull

struct JoinSmemLayout
{
  uint32_t size, bloom_words, exprs, staged;
  uint32_t nsum, nmin, nmax;
  uint32_t slot_of;                               // per expression (4 bits each): its index among its kind
  uint32_t keys, trows, bloom, cnt, lo, hi, mins, maxs, total;   // byte offsets in dynamic shared memory
};

__host__ __device__ inline JoinSmemLayout join_smem_layout(uint32_t size, uint32_t bloom_words, uint32_t exprs, uint32_t funcs,
                                                           bool staged)
{
  JoinSmemLayout l;
  l.size = size;
  l.bloom_words = bloom_words;
  l.exprs = exprs;
  l.staged = staged ? 1u : 0u;
  l.nsum = l.nmin = l.nmax = 0;
  l.slot_of = 0;
  for (uint32_t e = 0; e < exprs; e++)
  {
    uint32_t f = (funcs >> (4 * e)) & 0xfu, k = 0;
    if (f == 1u || f == 2u) k = l.nsum++;          // SUM, AVG
    else if (f == 3u) k = l.nmin++;               // MIN
    else if (f == 4u) k = l.nmax++;               // MAX
    l.slot_of |= k << (4 * e);
  }
  uint32_t off = 16;                              // the mbarrier sits in the first 8 bytes
  l.keys = off;
  if (staged) off += 4 * size;
  l.trows = off;
  if (staged) off += 4 * size;
  l.bloom = off;
  if (staged) off += 4 * bloom_words;
  l.cnt = off;
  off += 4 * size;
  l.lo = off;
  off += 4 * size * l.nsum;
  l.hi = off;
  off += 4 * size * l.nsum;
  l.mins = off;
  off += 4 * size * l.nmin;
  l.maxs = off;
  off += 4 * size * l.nmax;
  l.total = off;
  return l;
}

__device__ __forceinline__ uint64_t join_globaltimer()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// waits for phase 0 of the mbarrier for at most JOIN_WAIT_NS; 1 when it completed
__device__ __forceinline__ int join_mbar_wait(uint32_t bar)
{
  uint64_t t0 = join_globaltimer();
  for (;;)
  {
    uint32_t done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done) : "r"(bar), "r"(0u) : "memory");
    if (done) return 1;
    if (join_globaltimer() - t0 > JOIN_WAIT_NS) return 0;
  }
}

template <bool PLAIN, bool TSMEM>
__global__ void __launch_bounds__(JOIN_SMEM_THREADS, 2) k_join_probe_native_smem(CqlLaunch a, uint64_t rows, JoinSmemLayout L)
{
  extern __shared__ __align__(16) unsigned char smem[];
  JoinDecode d;
  uint32_t widths = cql_word(a, 1);
  uint32_t arg_base[4] = { cql_word(a, 3), cql_word(a, 5), cql_word(a, 9), cql_word(a, 11) };
#pragma unroll
  for (int c = 0; c < 5; c++)
  {
    uint32_t w = (widths >> (4 * c)) & 0xfu;
    d.col[c] = (const uint32_t*)a.buf[c];
    d.log2w[c] = w == 1 ? 2 : (w == 2 ? 1 : 0);
    d.bits[c] = w == 1 ? 8 : (w == 2 ? 16 : 32);
    d.mask[c] = w == 1 ? 0xffu : (w == 2 ? 0xffffu : 0xffffffffu);
    d.base[c] = (w == 1 || w == 2) ? (c == 0 ? cql_word(a, 10) : arg_base[c - 1]) : 0u;
  }
  uint32_t* counts = (uint32_t*)a.buf[7];
  unsigned long long* sums = (unsigned long long*)a.buf[8];
  int* mins = (int*)a.buf[9];
  int* maxs = (int*)a.buf[10];
  uint32_t* error = (uint32_t*)a.buf[12];
  const uint32_t exprs = L.exprs, funcs = cql_word(a, 4), arg_index = cql_word(a, 6), arg_signed = cql_word(a, 7);
  const uint32_t mask = L.size - 1u, log2_size = cql_word(a, 12), bloom_log2 = cql_word(a, 13);
  uint32_t used_args = 0;   // the argument columns some aggregate reads
  for (uint32_t e = 0; e < exprs; e++)
    if (((funcs >> (e * 4)) & 0xfu) != JFUNC_COUNT) used_args |= 1u << ((arg_index >> (e * 4)) & 0x3u);
  const uint64_t count_cap = a.bytes[7] / 4;
  const uint32_t* s_keys = TSMEM ? (const uint32_t*)(smem + L.keys) : (const uint32_t*)a.buf[5];
  const uint32_t* s_rows = TSMEM ? (const uint32_t*)(smem + L.trows) : (const uint32_t*)a.buf[6];
  const uint32_t* s_bloom = TSMEM ? (const uint32_t*)(smem + L.bloom) : (const uint32_t*)a.buf[11];
  uint32_t* s_cnt = (uint32_t*)(smem + L.cnt);
  // 64-bit sums as two 32-bit halves: a 32-bit shared atomic add, and a carry into the high half when the
  // low half wraps (or the value is negative), instead of a 64-bit shared atomic
  uint32_t* s_lo = (uint32_t*)(smem + L.lo);
  uint32_t* s_hi = (uint32_t*)(smem + L.hi);
  int* s_mins = (int*)(smem + L.mins);
  int* s_maxs = (int*)(smem + L.maxs);
  const uint32_t bar = (uint32_t)__cvta_generic_to_shared(smem);

  // stage the table and the Bloom words: one thread arms the barrier with the bytes and issues the copies
  if (TSMEM && threadIdx.x == 0)
  {
    uint32_t table_bytes = 4u * L.size, bloom_bytes = 4u * L.bloom_words;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(2u * table_bytes + bloom_bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(bar + L.keys), "l"(a.buf[5]), "r"(table_bytes), "r"(bar) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(bar + L.trows), "l"(a.buf[6]), "r"(table_bytes), "r"(bar) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(bar + L.bloom), "l"(a.buf[11]), "r"(bloom_bytes), "r"(bar) : "memory");
  }
  // the totals start empty while the copies fly
  for (uint32_t i = threadIdx.x; i < L.size; i += blockDim.x) s_cnt[i] = 0u;
  for (uint32_t i = threadIdx.x; i < L.size * L.nsum; i += blockDim.x)
  {
    s_lo[i] = 0u;
    s_hi[i] = 0u;
  }
  for (uint32_t i = threadIdx.x; i < L.size * L.nmin; i += blockDim.x) s_mins[i] = 0x7fffffff;
  for (uint32_t i = threadIdx.x; i < L.size * L.nmax; i += blockDim.x) s_maxs[i] = (int)0x80000000;
  __syncthreads();
  if (TSMEM && !join_mbar_wait(bar))
  {
    if (threadIdx.x == 0) atomicOr(error, 1u);
    join_mbar_wait(bar);      // the copies in flight land before the CTA leaves
    return;
  }

  const uint32_t UNROLL = 8;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; base < rows; base += stride * UNROLL)
  {
    uint32_t key[UNROLL];
    bool maybe[UNROLL];
#pragma unroll
    for (uint32_t u = 0; u < UNROLL; u++)
    {
      uint64_t at = base + u * stride;
      key[u] = at < rows ? join_read_t<PLAIN>(d, 0, at) : 0u;
    }
#pragma unroll
    for (uint32_t u = 0; u < UNROLL; u++)
    {
      uint64_t at = base + u * stride;
      uint32_t h = key[u] * 0x9E3779B1u, h2 = key[u] * 0x85EBCA6Bu;
      uint32_t bits = (1u << ((h2 >> 27) & 31u)) | (1u << ((h2 >> 22) & 31u));
      maybe[u] = at < rows && (s_bloom[h >> (32u - bloom_log2)] & bits) == bits;
    }
    // the argument words of every candidate row are loaded before the probes: their loads are in flight
    // together, and the probes and totals that follow touch shared memory (or L2) only
    uint32_t argv[UNROLL][4];
#pragma unroll
    for (uint32_t u = 0; u < UNROLL; u++)
#pragma unroll
      for (uint32_t c = 0; c < 4; c++) argv[u][c] = (maybe[u] && ((used_args >> c) & 1u)) ? join_read_t<PLAIN>(d, 1 + (int)c, base + u * stride) : 0u;
#pragma unroll
    for (uint32_t u = 0; u < UNROLL; u++)
    {
      if (!maybe[u]) continue;
      uint32_t slot = (key[u] * 0x9E3779B1u) >> (32u - log2_size);
      bool found = false;
      for (uint32_t probe = 0; probe < L.size; probe++)
      {
        uint32_t r1 = s_rows[slot];
        if (r1 == 0u) break;
        if (s_keys[slot] == key[u])
        {
          found = true;
          break;
        }
        slot = (slot + 1u) & mask;
      }
      if (!found) continue;
      atomicAdd(&s_cnt[slot], 1u);
      for (uint32_t e = 0; e < exprs; e++)
      {
        uint32_t f = (funcs >> (e * 4)) & 0xfu;
        if (f == JFUNC_COUNT) continue;
        uint32_t ai = (arg_index >> (e * 4)) & 0x3u;
        uint32_t w = ai == 0u ? argv[u][0] : ai == 1u ? argv[u][1] : ai == 2u ? argv[u][2] : argv[u][3];
        uint32_t index = ((L.slot_of >> (4 * e)) & 0xfu) * L.size + slot;
        if (f == JFUNC_SUM || f == JFUNC_AVG)
        {
          bool sg = ((arg_signed >> ai) & 1u) != 0;
          uint32_t old = atomicAdd(&s_lo[index], w);
          uint32_t up = ((sg && (int)w < 0) ? 0xffffffffu : 0u) + ((old + w < old) ? 1u : 0u);
          if (up) atomicAdd(&s_hi[index], up);
        }
        else if (f == JFUNC_MIN) atomicMin(&s_mins[index], (int)w);
        else if (f == JFUNC_MAX) atomicMax(&s_maxs[index], (int)w);
      }
    }
  }
  __syncthreads();
  // the CTA's totals per slot into the dim-row arrays
  for (uint32_t slot = threadIdx.x; slot < L.size; slot += blockDim.x)
  {
    uint32_t c = s_cnt[slot];
    if (c == 0u) continue;
    uint32_t dim_row = s_rows[slot] - 1u;
    if (dim_row >= count_cap) continue;
    atomicAdd(&counts[dim_row], c);
    for (uint32_t e = 0; e < exprs; e++)
    {
      uint32_t f = (funcs >> (e * 4)) & 0xfu;
      uint64_t index = (uint64_t)dim_row * exprs + e;
      uint32_t si = ((L.slot_of >> (4 * e)) & 0xfu) * L.size + slot;
      if (f == JFUNC_SUM || f == JFUNC_AVG) atomicAdd(&sums[index], ((unsigned long long)s_hi[si] << 32) | s_lo[si]);
      else if (f == JFUNC_MIN) atomicMin(&mins[index], s_mins[si]);
      else if (f == JFUNC_MAX) atomicMax(&maxs[index], s_maxs[si]);
    }
  }
}

static int launch_join_probe_native(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = cql_word(a, 0);
  uint32_t log2_size = cql_word(a, 12), bloom_log2 = cql_word(a, 13);
  if (rows == 0) return 0;
  if (log2_size == 0 || log2_size > 31 || bloom_log2 == 0 || bloom_log2 > 31) return (int)cudaErrorInvalidValue;
  if ((uint64_t)(cql_word(a, 8)) + 1 != (1ull << log2_size)) return (int)cudaErrorInvalidValue;
  // a small build side: the totals per slot in shared memory, and the table with them when it fits (the bulk
  // copies' sources and sizes are 16-byte multiples: tables of at least 16 slots and 16 Bloom words)
  uint32_t exprs = min(cql_word(a, 2), 8u);
  if (log2_size >= 4 && log2_size <= 16 && bloom_log2 >= 4 && bloom_log2 <= 16 && a.buf[12] && a.bytes[12] >= 4 &&
      ((uintptr_t)a.buf[5] & 15u) == 0 && ((uintptr_t)a.buf[6] & 15u) == 0 && ((uintptr_t)a.buf[11] & 15u) == 0 &&
      a.bytes[5] >= (4ull << log2_size) && a.bytes[6] >= (4ull << log2_size) && a.bytes[11] >= (4ull << bloom_log2))
  {
    uint32_t funcs = cql_word(a, 4);
    JoinSmemLayout L = join_smem_layout(1u << log2_size, 1u << bloom_log2, exprs, funcs, true);
    if (L.total > JOIN_SMEM_MAX_BYTES) L = join_smem_layout(1u << log2_size, 1u << bloom_log2, exprs, funcs, false);
    if (L.total <= JOIN_SMEM_MAX_BYTES && L.total <= (uint32_t)g_cql_max_smem_optin)
    {
      static bool attr_set = false;
      if (!attr_set)
      {
        const void* fns[4] = { (const void*)k_join_probe_native_smem<true, true>, (const void*)k_join_probe_native_smem<false, true>,
                               (const void*)k_join_probe_native_smem<true, false>, (const void*)k_join_probe_native_smem<false, false> };
        for (const void* fn : fns)
          if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min<uint32_t>(JOIN_SMEM_MAX_BYTES, (uint32_t)g_cql_max_smem_optin)) !=
              cudaSuccess)
            return (int)cudaGetLastError();
        attr_set = true;
      }
      bool plain = (cql_word(a, 1) & 0xfffffu) == 0u;   // key and every argument at full width
      // two CTAs an SM where their shared arrays fit (the register budget is set for two), else one
      int per_sm = L.total <= JOIN_SMEM_TWO_CTAS ? 2 : 1;
      dim3 grid(cql_stream_grid((rows + JOIN_SMEM_THREADS * 8 - 1) / (JOIN_SMEM_THREADS * 8), per_sm));
      if (L.staged)
      {
        if (plain) k_join_probe_native_smem<true, true><<<grid, JOIN_SMEM_THREADS, L.total, stream>>>(a, rows, L);
        else k_join_probe_native_smem<false, true><<<grid, JOIN_SMEM_THREADS, L.total, stream>>>(a, rows, L);
      }
      else
      {
        if (plain) k_join_probe_native_smem<true, false><<<grid, JOIN_SMEM_THREADS, L.total, stream>>>(a, rows, L);
        else k_join_probe_native_smem<false, false><<<grid, JOIN_SMEM_THREADS, L.total, stream>>>(a, rows, L);
      }
      CQL_LAUNCH_CHECK();
      return 0;
    }
  }
  k_join_probe_native<<<cql_stream_grid((rows + JOIN_THREADS * 8 - 1) / (JOIN_THREADS * 8), 3), JOIN_THREADS, 0, stream>>>(a, rows);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// Join-aggregate through a lookup table over the fact key's range (not a reference kernel: the
// reference probes a hash table of the dim keys and visits every dim row on the host,
// qe_aggregate_join_pushdown query_exec.c:8442-8776). With unique dim keys, each fact key value maps to
// at most one dim row and so to one group: the table turns the fact key column into a column of group
// ids that the dense group-by aggregates, and the first kept dim row of each group (its place in the
// output) is found on the device too. Key offsets are taken in 32-bit arithmetic (key - min mod 2^32),
// right for U32 and I32 keys alike; a key outside [min, min + range) matches nothing.
//
//  cql_join_lut_build  binding 0 visits (u32 dim rows; unbound: rows 0..visits-1), 1 dim keys (u32), 2 dim
//                      group values (word 12's type), 3 table (u32 group id per key value, all EMPTY before),
//                      4 visit per key value (u32), 5 error word; word 0 visits, word 2 1 = visit list
//                      given, word 4 min key bits, word 6 range, word 8/9 the smallest group value (f64
//                      bits), word 10 group values given (else every row is group 0), word 12 the group
//                      values' type (4 f64, 1 u32, 7 i32; 0 taken as f64).
//                      Error bit 0: a key met twice (the table cannot stand for the join).
//  cql_join_lut_map    binding 0 fact keys, 1 table, 2 group ids out (u32), 3 key-present bitmap (all 0
//                      before); word 0 rows, word 4 min key bits, word 6 range, word 8 the id of no group
//  cql_join_lut_first  binding 0 key-present bitmap, 1 table, 2 visit per key value, 3 first visit per
//                      group (u32, all EMPTY before); word 6 range

#define LUT_EMPTY 0xffffffffu

__global__ void __launch_bounds__(JOIN_THREADS) k_join_lut_build(CqlLaunch a, uint64_t visits)
{
  const uint32_t* visit_rows = (const uint32_t*)a.buf[0];
  const uint32_t* dim_keys = (const uint32_t*)a.buf[1];
  const double* group_values = (const double*)a.buf[2];
  const uint32_t* group_words = (const uint32_t*)a.buf[2];
  uint32_t* table = (uint32_t*)a.buf[3];
  uint32_t* visit_of = (uint32_t*)a.buf[4];
  uint32_t* error = (uint32_t*)a.buf[5];
  bool listed = cql_word(a, 2) != 0, grouped = cql_word(a, 10) != 0;
  uint32_t min_key = cql_word(a, 4), range = cql_word(a, 6);
  uint32_t group_type = cql_word(a, 12);    // 4 f64 (or 0), 1 u32, 7 i32
  bool group_f64 = group_type != 1u && group_type != 7u;
  double group_min = __longlong_as_double((long long)a.push[4]);
  uint64_t dim_rows = a.bytes[1] / 4, value_rows = a.bytes[2] / (group_f64 ? 8 : 4);
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < visits; v += (uint64_t)gridDim.x * blockDim.x)
  {
    uint64_t row = listed ? visit_rows[v] : v;
    if (row >= dim_rows || (grouped && row >= value_rows)) continue;
    uint32_t k = dim_keys[row] - min_key;
    if (k >= range) continue;
    double value = !grouped ? 0.0 : group_f64 ? group_values[row] : group_type == 7u ? (double)(int)group_words[row] : (double)group_words[row];
    uint32_t gid = grouped ? (uint32_t)(value - group_min) : 0u;
    uint32_t prev = atomicCAS(&table[k], LUT_EMPTY, gid);
    if (prev != LUT_EMPTY) atomicOr(error, 1u);
    else visit_of[k] = (uint32_t)v;
  }
}

__global__ void __launch_bounds__(JOIN_THREADS) k_join_lut_map(CqlLaunch a, uint64_t rows)
{
  const uint32_t* keys = (const uint32_t*)a.buf[0];
  const uint32_t* table = (const uint32_t*)a.buf[1];
  uint32_t* ids = (uint32_t*)a.buf[2];
  uint32_t* present = (uint32_t*)a.buf[3];
  uint32_t min_key = cql_word(a, 4), range = cql_word(a, 6), none = cql_word(a, 8);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t k = keys[i] - min_key;
    uint32_t gid = k < range ? table[k] : LUT_EMPTY;
    ids[i] = gid == LUT_EMPTY ? none : gid;
    if (gid != LUT_EMPTY)
    {
      // most keys repeat: read the word first, write it only the first time
      uint32_t bit = 1u << (k & 31u);
      if (!(present[k >> 5] & bit)) atomicOr(&present[k >> 5], bit);
    }
  }
}

__global__ void __launch_bounds__(JOIN_THREADS) k_join_lut_first(CqlLaunch a, uint64_t range)
{
  const uint32_t* present = (const uint32_t*)a.buf[0];
  const uint32_t* table = (const uint32_t*)a.buf[1];
  const uint32_t* visit_of = (const uint32_t*)a.buf[2];
  uint32_t* first = (uint32_t*)a.buf[3];
  uint64_t groups = a.bytes[3] / 4;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < range; k += (uint64_t)gridDim.x * blockDim.x)
  {
    if (!((present[k >> 5] >> (k & 31)) & 1u)) continue;
    uint32_t gid = table[k];
    // a group's first visit only falls: the atomic only when a plain read shows it larger (many keys
    // share few groups, and their atomics would serialise on them)
    uint32_t v = visit_of[k];
    if (gid < groups && v < __ldcg(&first[gid])) atomicMin(&first[gid], v);
  }
}

static int launch_join_lut_build(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t visits = cql_word(a, 0);
  uint64_t range = cql_word(a, 6);
  if (visits == 0) return 0;
  if (a.bytes[3] < range * 4 || a.bytes[4] < range * 4 || a.bytes[5] < 4 || (cql_word(a, 2) && a.bytes[0] < visits * 4))
    return (int)cudaErrorInvalidValue;
  k_join_lut_build<<<cql_stream_grid((visits + JOIN_THREADS - 1) / JOIN_THREADS, 8), JOIN_THREADS, 0, stream>>>(a, visits);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_join_lut_map(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = cql_word(a, 0);
  uint64_t range = cql_word(a, 6);
  if (rows == 0) return 0;
  if (a.bytes[0] < rows * 4 || a.bytes[1] < range * 4 || a.bytes[2] < rows * 4 || a.bytes[3] < ((range + 31) / 32) * 4)
    return (int)cudaErrorInvalidValue;
  k_join_lut_map<<<cql_stream_grid((rows + JOIN_THREADS - 1) / JOIN_THREADS, 8), JOIN_THREADS, 0, stream>>>(a, rows);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_join_lut_first(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t range = cql_word(a, 6);
  if (range == 0) return 0;
  if (a.bytes[0] < ((range + 31) / 32) * 4 || a.bytes[1] < range * 4 || a.bytes[2] < range * 4) return (int)cudaErrorInvalidValue;
  k_join_lut_first<<<cql_stream_grid((range + JOIN_THREADS - 1) / JOIN_THREADS, 8), JOIN_THREADS, 0, stream>>>(a, range);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// cql_join_dim_fold: the join-aggregate's dim-row pass on the device (not a reference kernel: the
// reference visits the dim rows on the host, qe_aggregate_join_pushdown query_exec.c:8619-8720). Each
// kept dim row whose key has fact rows adds its key's dense totals into its group's slot (the group value
// minus the smallest, or slot 0 without a GROUP BY) and leaves its visit number as the slot's first visit
// when it is the smallest: the host then orders the groups by first visit, as the host pass does.
//  binding 0 visits (u32 dim rows; unbound: rows 0..visits-1), 1 dim keys (u32), 2 dim group values (u32 or
//  i32 bits; unbound: no GROUP BY), 3 dense info (u32 pairs, word 1 the count), 4 dense sums (u32 lo/hi per
//  key and expression), 5 dense MIN, 6 dense MAX (i32 per key and expression), 7 slot counts (u64), 8 slot
//  sums (u64), 9 slot MIN, 10 slot MAX (i32), 11 slot first visit (u32, all 0xffffffff before)
//  words 0 visits, 2 1 = visit list given, 4 min key bits, 6 key range, 8 expressions, 10 smallest group value
//  bits, 12 slots, 14 bit 0 grouped, bit 1 MIN/MAX wanted

__global__ void __launch_bounds__(JOIN_THREADS) k_join_dim_fold(CqlLaunch a, uint64_t visits)
{
  const uint32_t* visit_rows = (const uint32_t*)a.buf[0];
  const uint32_t* dim_keys = (const uint32_t*)a.buf[1];
  const uint32_t* group_values = (const uint32_t*)a.buf[2];
  const uint32_t* info = (const uint32_t*)a.buf[3];
  const uint32_t* dsums = (const uint32_t*)a.buf[4];
  const int* dmins = (const int*)a.buf[5];
  const int* dmaxs = (const int*)a.buf[6];
  unsigned long long* counts = (unsigned long long*)a.buf[7];
  unsigned long long* sums = (unsigned long long*)a.buf[8];
  int* mins = (int*)a.buf[9];
  int* maxs = (int*)a.buf[10];
  uint32_t* first = (uint32_t*)a.buf[11];
  bool listed = cql_word(a, 2) != 0;
  uint32_t min_key = cql_word(a, 4), range = cql_word(a, 6), exprs = min(cql_word(a, 8), 8u), group_min = cql_word(a, 10);
  uint32_t slots = cql_word(a, 12), flags = cql_word(a, 14);
  bool grouped = (flags & 1u) != 0, want_mm = (flags & 2u) != 0;
  uint64_t dim_rows = a.bytes[1] / 4, value_rows = a.bytes[2] / 4;
  for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < visits; v += (uint64_t)gridDim.x * blockDim.x)
  {
    uint64_t row = listed ? visit_rows[v] : v;
    if (row >= dim_rows || (grouped && row >= value_rows)) continue;
    uint32_t id = dim_keys[row] - min_key;
    if (id >= range) continue;
    uint32_t n = info[2ull * id + 1];
    if (n == 0u) continue;
    uint32_t slot = grouped ? group_values[row] - group_min : 0u;
    if (slot >= slots) continue;
    atomicAdd(&counts[slot], (unsigned long long)n);
    for (uint32_t e = 0; e < exprs; e++)
    {
      uint64_t k = (uint64_t)id * exprs + e, s = (uint64_t)slot * exprs + e;
      atomicAdd(&sums[s], ((unsigned long long)dsums[2 * k + 1] << 32) | dsums[2 * k]);
      if (want_mm)
      {
        atomicMin(&mins[s], dmins[k]);
        atomicMax(&maxs[s], dmaxs[k]);
      }
    }
    atomicMin(&first[slot], (uint32_t)v);
  }
}

static int launch_join_dim_fold(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t visits = cql_word(a, 0);
  if (visits == 0) return 0;
  k_join_dim_fold<<<cql_stream_grid((visits + JOIN_THREADS - 1) / JOIN_THREADS, 8), JOIN_THREADS, 0, stream>>>(a, visits);
  CQL_LAUNCH_CHECK();
  return 0;
}

const CqlKernelDesc cql_kernels_join[] = {
  { "hash_join_build_count", launch_join_build_count },
  { "prefix_sum", launch_prefix_sum },
  { "prefix_sum2", launch_prefix_sum },
  { "hash_join_probe", launch_join_probe },
  { "join_pack_key", launch_join_pack_key },
  { "join_probe_native", launch_join_probe_native },
  { "cql_join_lut_build", launch_join_lut_build },
  { "cql_join_lut_map", launch_join_lut_map },
  { "cql_join_lut_first", launch_join_lut_first },
  { "cql_join_dim_fold", launch_join_dim_fold },
  { nullptr, nullptr },
};
