// Hash GROUP BY: slot assignment, compaction, atomic reduce, member lists, member reduce with the
// HyperLogLog and t-digest sketches, and the selection gather.
//
//  aggregate_assign            src/gpu/vulkan/shaders/aggregate_assign.comp:1-186
//  aggregate_compact           src/gpu/vulkan/shaders/aggregate_compact.comp:1-111
//  aggregate_hash_reduce_fixed src/gpu/vulkan/shaders/aggregate_hash_reduce_fixed.comp:1-122
//  csr_scatter / _tiled        src/gpu/vulkan/shaders/csr_scatter.comp:1-31, csr_scatter_tiled.comp:1-77
//  aggregate_reduce            src/gpu/vulkan/shaders/aggregate_reduce.comp:1-222
//  selection_gather            src/gpu/vulkan/shaders/selection_gather.comp:1-78
//
// The slot table is buckets x K slots whose owner row is claimed with a compare-and-swap, keys are
// compared as f64 values (or string bytes) and hashed from their bit patterns; the HyperLogLog
// register update hashes the f64 bit pattern of each value the same way (hash_u32(lo ^ hash_u32(hi)),
// bucket = top p bits, rho = position of the leading one of the rest), so the registers are
// identical to the reference's for the same values. GB300 design: persistent grid-stride launches
// instead of one thread per row, and the member reduce runs one warp per chunk (eight of the
// reference's 256 lanes per warp lane) so groups of a few rows do not idle 256 threads each, while
// the per-lane t-digest centroid (first sample, weight) is computed for the same 256 lane positions.
#include "cql_internal.cuh"
#include "cql_fixed.cuh"
#include <algorithm>
#include <float.h>
#include <string.h>

#define HASH_THREADS 256
#define EMPTY_SLOT 0xffffffffu
#define PAST_END 0xfffffffeu

__device__ __forceinline__ uint32_t hash_u32(uint32_t x)
{
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// ---------------------------------------------------------------------------------------------
// aggregate_assign: binding 0 owner row per slot, 1 rows per slot, 2 slot per row, 3 overflow count,
// 4 + 2c / 5 + 2c key column c (f64 values, or string bytes + u64 offsets);
// words 0 rows, 2 buckets, 4 K, 6 key columns, 8 string mask, 10 1 = count atomics per lane (many groups),
// 12 1 = linear probing over the whole table (slots a power of two), 14 per key column 4 bits: its CQL type
// when it is bound at its stored width (U32, I32, F32), widened to f64 in registers; 0 = f64 values (the
// reference's layout)

struct KeyCols
{
  const uint32_t* data[4];
  const uint32_t* off[4];
  uint32_t types;
};

// a numeric key's f64 value and its bits, from the f64 pairs or the stored width
__device__ __forceinline__ double key_value(const KeyCols& k, uint32_t c, uint64_t row)
{
  uint32_t t = (k.types >> (4 * c)) & 0xfu;
  if (t == 0u) return __hiloint2double((int)k.data[c][row * 2 + 1], (int)k.data[c][row * 2]);
  return cql_value_as_f64(k.data[c], t, row);
}

__device__ __forceinline__ uint32_t key_str_off(const KeyCols& k, uint32_t c, uint64_t row) { return k.off[c][row * 2]; }
__device__ __forceinline__ uint32_t key_byte(const KeyCols& k, uint32_t c, uint64_t i) { return ((const unsigned char*)k.data[c])[i]; }

__device__ uint32_t key_hash(const KeyCols& k, uint32_t ncols, uint32_t string_mask, uint64_t row)
{
  uint32_t h = 2166136261u;
  for (uint32_t c = 0; c < ncols; c++)
  {
    uint32_t hh;
    if ((string_mask >> c) & 1u)
    {
      uint32_t s = key_str_off(k, c, row), e = key_str_off(k, c, row + 1);
      hh = 2166136261u;
      for (uint32_t i = s; i < e; i++) hh = (hh ^ key_byte(k, c, i)) * 16777619u;
    }
    else
    {
      unsigned long long bits = (unsigned long long)__double_as_longlong(key_value(k, c, row));
      uint32_t lo = (uint32_t)bits, hi = (uint32_t)(bits >> 32);
      hh = hash_u32(lo ^ hash_u32(hi));
    }
    h = hash_u32(h ^ hh);
  }
  return h;
}

__device__ bool keys_equal(const KeyCols& k, uint32_t ncols, uint32_t string_mask, uint64_t a, uint64_t b)
{
  for (uint32_t c = 0; c < ncols; c++)
  {
    if ((string_mask >> c) & 1u)
    {
      uint32_t sa = key_str_off(k, c, a), ea = key_str_off(k, c, a + 1);
      uint32_t sb = key_str_off(k, c, b), eb = key_str_off(k, c, b + 1);
      if (ea - sa != eb - sb) return false;
      for (uint32_t i = 0; i < ea - sa; i++)
        if (key_byte(k, c, sa + i) != key_byte(k, c, sb + i)) return false;
    }
    else
    {
      double x = key_value(k, c, a), y = key_value(k, c, b);
      if (!(x == y)) return false;
    }
  }
  return true;
}

// The lanes of the warp that share this lane's tag, for one atomic per distinct tag. With many groups
// (alone: the host knows or was told there are thousands) a warp's lanes almost never share one, and a
// lane's own atomic costs less than the match instruction that would find its peers.
__device__ __forceinline__ uint32_t combine_peers(uint32_t tag, bool alone, uint32_t lane)
{
  return alone ? (1u << lane) : __match_any_sync(0xffffffffu, tag);
}

__global__ void __launch_bounds__(HASH_THREADS) k_aggregate_assign(CqlLaunch a, uint64_t rows)
{
  uint32_t* owner = (uint32_t*)a.buf[0];
  uint32_t* counts = (uint32_t*)a.buf[1];
  uint32_t* row_slot = (uint32_t*)a.buf[2];
  uint32_t* overflow = (uint32_t*)a.buf[3];
  uint32_t buckets = cql_word(a, 2), K = cql_word(a, 4), ncols = cql_word(a, 6), string_mask = cql_word(a, 8);
  bool alone = cql_word(a, 10) != 0;
  // word 12: 1 = linear probing over the whole table (a power of two of slots): K probes from slot
  // hash mod slots, wrapping, instead of the K slots of the hash's bucket
  bool linear = cql_word(a, 12) != 0;
  if (ncols > 4) ncols = 4;
  KeyCols k;
  for (int c = 0; c < 4; c++)
  {
    k.data[c] = (const uint32_t*)a.buf[4 + 2 * c];
    k.off[c] = (const uint32_t*)a.buf[5 + 2 * c];
  }
  k.types = cql_word(a, 14);
  uint64_t slots = a.bytes[0] / 4;
  uint32_t lane = threadIdx.x & 31u;
  // the loop runs while the warp's first row is in range, so whole warps take every iteration together
  for (uint64_t row = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; row - lane < rows; row += (uint64_t)gridDim.x * blockDim.x)
  {
    bool valid = row < rows;
    uint32_t h = (valid && ncols) ? key_hash(k, ncols, string_mask, row) : 0u;
    uint64_t start = linear ? (uint64_t)h & (slots - 1) : (uint64_t)(h % (buckets ? buckets : 1u)) * K;
    uint32_t claimed = EMPTY_SLOT;
    for (uint32_t p = 0; valid && p < K; p++)
    {
      uint64_t slot = linear ? (start + p) & (slots - 1) : start + p;
      if (slot >= slots) break;
      // a slot's owner only ever goes from empty to a row: read it first, claim it only when empty
      uint32_t prev = *((volatile uint32_t*)&owner[slot]);
      if (prev == EMPTY_SLOT) prev = atomicCAS(&owner[slot], EMPTY_SLOT, (uint32_t)row);
      if (prev == EMPTY_SLOT || keys_equal(k, ncols, string_mask, row, prev))
      {
        claimed = (uint32_t)slot;
        break;
      }
    }
    if (valid && claimed != EMPTY_SLOT) row_slot[row] = claimed;
    // one count atomic per distinct slot of the warp (few groups would otherwise serialise on them)
    uint32_t tag = valid ? claimed : PAST_END;
    uint32_t peers = combine_peers(tag, alone, lane);
    if (lane == (uint32_t)(__ffs(peers) - 1) && tag != PAST_END)
    {
      if (claimed == EMPTY_SLOT) atomicAdd(overflow, (uint32_t)__popc(peers));
      else atomicAdd(&counts[claimed], (uint32_t)__popc(peers));
    }
  }
}

static int launch_aggregate_assign(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = cql_word(a, 0);
  if (rows == 0) return 0;
  k_aggregate_assign<<<cql_stream_grid((rows + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, rows);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// aggregate_compact: three modes over blocks of 256 slots (the block sums index is index / 256)

__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* sh, uint32_t* total)
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
    for (int w = 0; w < HASH_THREADS / 32; w++)
    {
      uint32_t t = sh[w];
      sh[w] = run;
      run += t;
    }
    sh[HASH_THREADS / 32] = run;
  }
  __syncthreads();
  uint32_t ex = sh[warp] + incl - v;
  *total = sh[HASH_THREADS / 32];
  __syncthreads();
  return ex;
}

__global__ void __launch_bounds__(HASH_THREADS) k_aggregate_compact(CqlLaunch a, uint32_t mode, uint32_t n)
{
  __shared__ uint32_t sh[HASH_THREADS / 32 + 1];
  const uint32_t* counts = (const uint32_t*)a.buf[0];
  const uint32_t* owner = (const uint32_t*)a.buf[1];
  uint32_t* offsets = (uint32_t*)a.buf[2];
  uint32_t* block_sums = (uint32_t*)a.buf[3];
  uint32_t* out_owner = (uint32_t*)a.buf[4];
  uint32_t* out_count = (uint32_t*)a.buf[5];
  uint32_t* total_out = (uint32_t*)a.buf[6];
  uint32_t blocks = (n + 255) / 256;
  uint32_t total;
  if (mode == 0)
  {
    for (uint32_t b = blockIdx.x; b < blocks; b += gridDim.x)
    {
      uint32_t index = b * 256 + threadIdx.x;
      uint32_t v = (index < n && counts[index] != 0) ? 1u : 0u;
      uint32_t ex = block_exclusive_scan(v, sh, &total);
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
    uint32_t running = block_exclusive_scan(sum, sh, &total);
    for (uint32_t i = start; i < end; i++)
    {
      uint32_t t = block_sums[i];
      block_sums[i] = running;
      running += t;
    }
    if (threadIdx.x == 0)
    {
      offsets[n] = total;
      total_out[0] = total;
    }
  }
  else
  {
    for (uint64_t index = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; index < n; index += (uint64_t)gridDim.x * blockDim.x)
    {
      uint32_t id = offsets[index] + block_sums[index / 256];
      offsets[index] = id;
      uint32_t c = counts[index];
      if (c != 0)
      {
        out_owner[id] = owner[index];
        out_count[id] = c;
      }
    }
  }
}

static int launch_aggregate_compact(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint32_t n = cql_word(a, 0), mode = cql_word(a, 2);
  uint32_t blocks = (n + 255) / 256;
  if (mode == 1) k_aggregate_compact<<<1, HASH_THREADS, 0, stream>>>(a, mode, n);
  else k_aggregate_compact<<<cql_stream_grid(blocks ? blocks : 1, 8), HASH_THREADS, 0, stream>>>(a, mode, n);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// Slot compaction that allocates nothing.
//
// Some callers cannot allocate device memory while they run a query. One example is a serving loop
// that reserves all of HBM ahead of time: it gives most of it to resident tables and sets aside a
// fixed budget for each admitted query. There, a cudaMalloc on the query path can fail, or can force
// an eviction halfway through a query. For those callers, this entry point runs the same three
// aggregate_compact passes with the block totals (the kernel's only scratch) in a static device
// array. Every GPU that loads this library holds that array until the process exits.
//
// Limit: CQL_NOALLOC_COMPACT_MAX_SLOTS slots (2^24, i.e. 65536 blocks of 256; 256 KB of scratch).
// The array's device address is looked up with cudaGetSymbolAddress, with the device current, once
// per device: by cqlcuda_init for the device it opens (which also loads the kernel, so that under
// lazy module loading no later call loads a module), else by the first call on a device. Make that
// first call before any stream capture. All calls share the array. Calls whose work overlaps on the
// GPU race on it: serialise them, for example by issuing them on one stream. Nothing in the array has
// to start at zero: every block total is written before it is read, and so is the group total.

#define CQL_NOALLOC_COMPACT_MAX_SLOTS (1u << 24)
#define CQL_NOALLOC_COMPACT_BLOCKS (CQL_NOALLOC_COMPACT_MAX_SLOTS / 256u)
#define CQL_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) uint32_t g_noalloc_compact_scratch[CQL_NOALLOC_COMPACT_BLOCKS + 64];

static uint32_t* g_noalloc_scratch_ptr[CQL_NOALLOC_MAX_DEVICES];

static int noalloc_resolve(int device)
{
  if (g_noalloc_scratch_ptr[device]) return 1;
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_compact_scratch) != cudaSuccess || !p) return 0;
  cudaFuncAttributes attr;
  if (cudaFuncGetAttributes(&attr, k_aggregate_compact) != cudaSuccess) return 0;
  g_noalloc_scratch_ptr[device] = (uint32_t*)p;
  return 1;
}

int cql_noalloc_prepare(void)
{
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= CQL_NOALLOC_MAX_DEVICES) return 0;
  return noalloc_resolve(device);
}

extern "C" int cqlcuda_compact_slots_noalloc(const uint32_t* slot_counts, const uint32_t* slot_owner, uint32_t slot_count,
                                             uint32_t* slot_group, uint32_t* group_owner, uint32_t* group_count, uint32_t* out_group_total,
                                             void* stream)
{
  if (slot_count == 0 || slot_count > CQL_NOALLOC_COMPACT_MAX_SLOTS)
  {
    cql_set_error_text("cqlcuda_compact_slots_noalloc: %u slots; it takes 1 to %u", slot_count, CQL_NOALLOC_COMPACT_MAX_SLOTS);
    return -1;
  }
  if (!slot_counts || !slot_owner || !slot_group || !group_owner || !group_count || !out_group_total)
  {
    cql_set_error_text("cqlcuda_compact_slots_noalloc: a NULL pointer argument");
    return -2;
  }
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= CQL_NOALLOC_MAX_DEVICES || !noalloc_resolve(device))
  {
    cql_set_error_text("cqlcuda_compact_slots_noalloc: no usable device (its static scratch could not be resolved)");
    return -3;
  }
  uint32_t* scratch = g_noalloc_scratch_ptr[device];
  cudaStream_t s = (cudaStream_t)stream;
  CqlLaunch a;
  memset(&a, 0, sizeof(a));
  uint32_t blocks = (slot_count + 255u) / 256u;
  a.buf[0] = (void*)slot_counts;
  a.bytes[0] = (uint64_t)slot_count * 4;
  a.buf[1] = (void*)slot_owner;
  a.bytes[1] = (uint64_t)slot_count * 4;
  a.buf[2] = slot_group;
  a.bytes[2] = ((uint64_t)slot_count + 1) * 4;
  a.buf[3] = scratch;                                  // block totals
  a.bytes[3] = (uint64_t)blocks * 4;
  a.buf[4] = group_owner;
  a.bytes[4] = (uint64_t)slot_count * 4;
  a.buf[5] = group_count;
  a.bytes[5] = (uint64_t)slot_count * 4;
  a.buf[6] = scratch + CQL_NOALLOC_COMPACT_BLOCKS;     // group total
  a.bytes[6] = 4;
  a.push[0] = slot_count;
  // an earlier, unrelated launch error still pending on this thread is not this call's failure
  (void)cudaGetLastError();
  for (uint32_t mode = 0; mode < 3; mode++)
  {
    a.push[1] = mode;
    if (mode == 1) k_aggregate_compact<<<1, HASH_THREADS, 0, s>>>(a, mode, slot_count);
    else k_aggregate_compact<<<cql_stream_grid(blocks, 8), HASH_THREADS, 0, s>>>(a, mode, slot_count);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
    {
      cql_set_error_text("cqlcuda_compact_slots_noalloc: launch of pass %u failed: %s", mode, cudaGetErrorString(e));
      return -4;
    }
    cql_note_launch();
  }
  cudaError_t e = cudaMemcpyAsync(out_group_total, scratch + CQL_NOALLOC_COMPACT_BLOCKS, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
  {
    cql_set_error_text("cqlcuda_compact_slots_noalloc: %s", cudaGetErrorString(e));
    return -4;
  }
  return 1;
}

// ---------------------------------------------------------------------------------------------
// aggregate_hash_reduce_fixed: binding 0 slot per row, 1 group per slot, 2 sums (lo, hi), 3 counts,
// 4 mins, 5 maxs, 6..13 f64 arguments; words 0 rows, 2 exprs, 4 funcs, 6 power-of-ten exponents,
// 8 1 = atomics per lane (many groups)

#define FUNC_COUNT 0u
#define FUNC_SUM 1u
#define FUNC_AVG 2u
#define FUNC_MIN 3u
#define FUNC_MAX 4u
#define FUNC_ACD 5u
#define FUNC_PCT 6u


__global__ void __launch_bounds__(HASH_THREADS) k_hash_reduce_fixed(CqlLaunch a, uint64_t rows)
{
  const uint32_t* row_slot = (const uint32_t*)a.buf[0];
  const uint32_t* slot_group = (const uint32_t*)a.buf[1];
  unsigned long long* sums = (unsigned long long*)a.buf[2];
  uint32_t* counts = (uint32_t*)a.buf[3];
  int* mins = (int*)a.buf[4];
  int* maxs = (int*)a.buf[5];
  uint32_t exprs = min(cql_word(a, 2), 8u), funcs = cql_word(a, 4), scales = cql_word(a, 6);
  bool alone = cql_word(a, 8) != 0;
  uint64_t nslots = a.bytes[1] / 4;
  uint32_t lane = threadIdx.x & 31u;
  // whole warps take every iteration, so the lanes of one group combine before a single atomic
  for (uint64_t row = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; row - lane < rows; row += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t g = PAST_END;
    if (row < rows)
    {
      uint32_t slot = row_slot[row];
      if (slot < nslots)
      {
        uint32_t gg = slot_group[slot];
        if (gg != EMPTY_SLOT) g = gg;
      }
    }
    uint32_t peers = combine_peers(g, alone, lane);
    bool leader = lane == (uint32_t)(__ffs(peers) - 1) && g != PAST_END;
    for (uint32_t e = 0; e < exprs; e++)
    {
      uint32_t f = (funcs >> (e * 4)) & 0xfu;
      uint64_t index = (uint64_t)g * exprs + e;
      if (leader) atomicAdd(&counts[index], (uint32_t)__popc(peers));
      if (f == FUNC_COUNT) continue;
      // floor(v * 10^s + 0.5) of the argument, in integer arithmetic (exact for decimals of scale s)
      int q = 0;
      if (g != PAST_END)
        q = fix_scaled(fix_decode_f64(((const unsigned long long*)a.buf[6 + e])[row]), (int)min((scales >> (e * 4)) & 0xfu, 6u));
      long long acc = q;
      int mn = q, mx = q;
      if (!alone)
      {
        acc = 0;
        mn = 0x7fffffff;
        mx = (int)0x80000000;
#pragma unroll 8
        for (int src = 0; src < 32; src++)
        {
          int v = __shfl_sync(0xffffffffu, q, src);
          if ((peers >> src) & 1u)
          {
            acc += v;
            mn = min(mn, v);
            mx = max(mx, v);
          }
        }
      }
      if (!leader) continue;
      if (f == FUNC_SUM || f == FUNC_AVG) atomicAdd(&sums[index], (unsigned long long)acc);
      else if (f == FUNC_MIN) atomicMin(&mins[index], mn);
      else if (f == FUNC_MAX) atomicMax(&maxs[index], mx);
    }
  }
}

static int launch_hash_reduce_fixed(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = cql_word(a, 0);
  if (rows == 0) return 0;
  k_hash_reduce_fixed<<<cql_stream_grid((rows + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, rows);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// csr_scatter (and the tiled variant, same bindings plus the slot count in slot 1): every row takes
// the next place of its slot's member list through the slot's cursor; word 0 rows, word 2 1 = one
// atomic per lane (many slots)

__global__ void __launch_bounds__(HASH_THREADS) k_csr_scatter(CqlLaunch a, uint64_t rows)
{
  const uint32_t* row_slot = (const uint32_t*)a.buf[0];
  uint32_t* cursor = (uint32_t*)a.buf[1];
  uint32_t* out_rows = (uint32_t*)a.buf[2];
  uint64_t cap = a.bytes[2] / 4, slots = a.bytes[1] / 4;
  bool alone = cql_word(a, 2) != 0;
  uint32_t lane = threadIdx.x & 31u;
  for (uint64_t row = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; row - lane < rows; row += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t slot = row < rows ? row_slot[row] : EMPTY_SLOT;
    if (slot >= slots) slot = EMPTY_SLOT;
    // lanes of one slot take consecutive places with one atomic
    uint32_t peers = combine_peers(slot, alone, lane);
    uint32_t leader = (uint32_t)(__ffs(peers) - 1);
    uint32_t base = 0;
    if (lane == leader && slot != EMPTY_SLOT) base = atomicAdd(&cursor[slot], (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    uint32_t pos = base + __popc(peers & ((1u << lane) - 1u));
    if (slot != EMPTY_SLOT && pos < cap) out_rows[pos] = (uint32_t)row;
  }
}

static int launch_csr_scatter(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = cql_word(a, 0);
  if (rows == 0) return 0;
  k_csr_scatter<<<cql_stream_grid((rows + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, rows);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// aggregate_reduce: chunk c covers members [range[2c], range[2c+1]) of group chunk_group[c].
// binding 0 members, 1 chunk ranges, 2 chunk groups, 3 representative per group, 4 partials
// [chunk][expr][acc, count, min, max], 5..12 f64 arguments, 13 HLL registers
// [group][hll expr][2^p], 14/15 t-digest centroid mean/weight [chunk][pct expr][256].
// words 0 chunks, 2 exprs, 4 funcs, 6 identity mode, 8 HLL precision, 10 HLL slot per expr,
// 12 HLL exprs, 14 percentile exprs, 15 percentile slot per expr

__device__ __forceinline__ void hll_add(uint32_t* sketch, uint64_t sketch_words, uint32_t slot, uint32_t g, uint32_t nhll, uint32_t p, double value)
{
  unsigned long long bits = (unsigned long long)__double_as_longlong(value);
  uint32_t lo = (uint32_t)bits, hi = (uint32_t)(bits >> 32);
  uint32_t h = hash_u32(lo ^ hash_u32(hi));
  uint32_t rest_bits = 32u - p;
  uint32_t bucket = h >> rest_bits;
  uint32_t rest = h & ((1u << rest_bits) - 1u);
  // findMSB: the index of the highest set bit, -1 for zero
  int msb = rest ? 31 - __clz(rest) : -1;
  uint32_t rho = msb < 0 ? rest_bits + 1u : rest_bits - (uint32_t)msb;
  uint64_t idx = ((uint64_t)g * nhll + slot) * (1ull << p) + bucket;
  // registers only grow: a value read at least as large (even a stale one) makes the atomic redundant,
  // and after the first rows almost every value is below its register
  if (idx < sketch_words && __ldcg(&sketch[idx]) < rho) atomicMax(&sketch[idx], rho);
}

struct ReduceArgs
{
  const uint32_t* members;
  uint32_t* repr;
  double* partials;
  uint32_t* sketch;
  float* dmean;
  float* dweight;
  uint64_t sketch_words, digest_cap, partial_cap;
  uint32_t exprs, funcs, p, hll_slots, nhll, npct, pct_slots;
  bool identity;
};

__device__ __forceinline__ void reduce_store(const ReduceArgs& r, uint32_t c, uint32_t e, double acc, uint32_t count, double mn, double mx)
{
  uint64_t base = ((uint64_t)c * r.exprs + e) * 4;
  if (base + 3 < r.partial_cap)
  {
    r.partials[base + 0] = acc;
    r.partials[base + 1] = (double)count;
    r.partials[base + 2] = mn;
    r.partials[base + 3] = mx;
  }
}

// One chunk by the whole warp, in the reference's layout: this lane stands for reference lanes
// t = lane + 32 j, j = 0..7, each taking members start + t, start + t + 256, ...; the t-digest's
// per-lane centroids (the first value and the count of each reference lane) need exactly this layout.
__device__ __forceinline__ void reduce_chunk_warp(const CqlLaunch& a, const ReduceArgs& r, uint32_t c, uint32_t start, uint32_t end, uint32_t g, uint32_t lane)
{
  if (lane == 0 && (r.identity || end > start)) r.repr[g] = r.identity ? start : r.members[start];
  for (uint32_t e = 0; e < r.exprs; e++)
  {
    uint32_t f = (r.funcs >> (e * 4)) & 0xfu;
    const double* arg = (const double*)a.buf[5 + e];
    double acc = 0.0, mn = 1.0e300, mx = -1.0e300;
    uint32_t count = 0;
    for (uint32_t j = 0; j < 8; j++)
    {
      uint32_t t = lane + 32 * j;
      double first = 0.0;
      uint32_t tcount = 0;
      for (uint32_t m = start + t; m < end; m += 256)
      {
        uint32_t row = r.identity ? m : r.members[m];
        tcount++;
        if (f == FUNC_SUM || f == FUNC_AVG) acc += arg[row];
        else if (f == FUNC_MIN) { double v = arg[row]; if (v < mn) mn = v; }
        else if (f == FUNC_MAX) { double v = arg[row]; if (v > mx) mx = v; }
        else if (f == FUNC_ACD) hll_add(r.sketch, r.sketch_words, (r.hll_slots >> (e * 4)) & 0xfu, g, r.nhll, r.p, arg[row]);
        else if (f == FUNC_PCT && tcount == 1) first = arg[row];
      }
      count += tcount;
      if (f == FUNC_PCT)
      {
        uint64_t di = ((uint64_t)c * r.npct + ((r.pct_slots >> (e * 4)) & 0xfu)) * 256u + t;
        if (di < r.digest_cap)
        {
          r.dmean[di] = (float)first;
          r.dweight[di] = (float)tcount;
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
      acc += __shfl_xor_sync(0xffffffffu, acc, o);
      double omn = __shfl_xor_sync(0xffffffffu, mn, o);
      double omx = __shfl_xor_sync(0xffffffffu, mx, o);
      mn = omn < mn ? omn : mn;
      mx = omx > mx ? omx : mx;
      count += __shfl_xor_sync(0xffffffffu, count, o);
    }
    if (lane == 0) reduce_store(r, c, e, acc, count, mn, mx);
  }
}

// One small chunk by one lane, its members in order: the same partials (sums in another order, within
// rounding of the warp's), for chunks of a few members, where the warp form spends most of its
// instructions on empty reference lanes and cross-lane reductions.
__device__ __forceinline__ void reduce_chunk_lane(const CqlLaunch& a, const ReduceArgs& r, uint32_t c, uint32_t start, uint32_t end, uint32_t g)
{
  if (r.identity || end > start) r.repr[g] = r.identity ? start : r.members[start];
  for (uint32_t e = 0; e < r.exprs; e++)
  {
    uint32_t f = (r.funcs >> (e * 4)) & 0xfu;
    const double* arg = (const double*)a.buf[5 + e];
    double acc = 0.0, mn = 1.0e300, mx = -1.0e300;
    if (f == FUNC_SUM || f == FUNC_AVG || f == FUNC_MIN || f == FUNC_MAX || f == FUNC_ACD)
      for (uint32_t m = start; m < end; m++)
      {
        uint32_t row = r.identity ? m : r.members[m];
        double v = arg[row];
        if (f == FUNC_SUM || f == FUNC_AVG) acc += v;
        else if (f == FUNC_MIN) { if (v < mn) mn = v; }
        else if (f == FUNC_MAX) { if (v > mx) mx = v; }
        else hll_add(r.sketch, r.sketch_words, (r.hll_slots >> (e * 4)) & 0xfu, g, r.nhll, r.p, v);
      }
    reduce_store(r, c, e, acc, end - start, mn, mx);
  }
}

#define REDUCE_LANE_CHUNK 64   // chunks of at most this many members are reduced by one lane

__global__ void __launch_bounds__(HASH_THREADS) k_aggregate_reduce(CqlLaunch a, uint32_t chunks)
{
  const uint32_t* range = (const uint32_t*)a.buf[1];
  const uint32_t* chunk_group = (const uint32_t*)a.buf[2];
  ReduceArgs r;
  r.members = (const uint32_t*)a.buf[0];
  r.repr = (uint32_t*)a.buf[3];
  r.partials = (double*)a.buf[4];
  r.sketch = (uint32_t*)a.buf[13];
  r.dmean = (float*)a.buf[14];
  r.dweight = (float*)a.buf[15];
  r.sketch_words = a.bytes[13] / 4;
  r.digest_cap = a.bytes[14] / 4;
  r.partial_cap = a.bytes[4] / 8;
  r.exprs = min(cql_word(a, 2), 8u);
  r.funcs = cql_word(a, 4);
  r.identity = cql_word(a, 6) != 0;
  r.p = min(cql_word(a, 8), 16u);
  r.hll_slots = cql_word(a, 10);
  r.nhll = cql_word(a, 12);
  r.npct = cql_word(a, 14);
  r.pct_slots = cql_word(a, 15);
  uint32_t lane = threadIdx.x & 31;
  uint32_t warps_total = gridDim.x * (blockDim.x / 32);
  uint32_t warp_id = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  // a warp takes 32 chunks spaced the grid's warp count apart: each lane reduces a small one alone,
  // then the warp reduces the large ones together (all of them when a percentile needs the reference's
  // lane layout); the spacing spreads a run of large chunks (one large group's) over many warps
  for (uint64_t first = warp_id; first < chunks; first += 32ull * warps_total)
  {
    uint64_t c = first + (uint64_t)lane * warps_total;
    uint32_t start = 0, end = 0, g = 0;
    bool have = c < chunks;
    if (have)
    {
      start = range[c * 2];
      end = range[c * 2 + 1];
      g = chunk_group[c];
    }
    bool alone = have && r.npct == 0 && end - start <= REDUCE_LANE_CHUNK;
    if (alone) reduce_chunk_lane(a, r, (uint32_t)c, start, end, g);
    uint32_t big = __ballot_sync(0xffffffffu, have && !alone);
    while (big)
    {
      uint32_t src = (uint32_t)(__ffs(big) - 1);
      big &= big - 1;
      uint32_t bs = __shfl_sync(0xffffffffu, start, src), be = __shfl_sync(0xffffffffu, end, src), bg = __shfl_sync(0xffffffffu, g, src);
      reduce_chunk_warp(a, r, (uint32_t)(first + (uint64_t)src * warps_total), bs, be, bg, lane);
    }
  }
}

static int launch_aggregate_reduce(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint32_t chunks = cql_word(a, 0);
  if (chunks == 0) return 0;
  // a warp per chunk up to the resident grid (the large chunks' parallelism), 32 chunks a warp beyond
  uint32_t warps = HASH_THREADS / 32;
  k_aggregate_reduce<<<cql_stream_grid((chunks + warps - 1) / warps, 8), HASH_THREADS, 0, stream>>>(a, chunks);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// selection_gather: binding 0 rows (one index every `stride` words), 1 source, 2 destination,
// 3 positions; words 0 count, 2 stride, 4 row offset, 6 mode, 8 map stride, 10 word offset, 12 map offset

__global__ void __launch_bounds__(HASH_THREADS) k_selection_gather(CqlLaunch a, uint64_t count)
{
  const uint32_t* rows = (const uint32_t*)a.buf[0];
  const uint32_t* source = (const uint32_t*)a.buf[1];
  uint32_t* dest = (uint32_t*)a.buf[2];
  const uint32_t* positions = (const uint32_t*)a.buf[3];
  uint32_t stride = cql_word(a, 2), row_offset = cql_word(a, 4), mode = cql_word(a, 6);
  uint32_t map_stride = cql_word(a, 8), word_offset = cql_word(a, 10), map_offset = cql_word(a, 12);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x)
  {
    if (mode == 2)
    {
      uint32_t index = rows[(uint64_t)positions[i] * stride + word_offset];
      dest[i] = index == EMPTY_SLOT ? EMPTY_SLOT : index + row_offset;
      continue;
    }
    uint32_t index = rows[i * stride + word_offset];
    if (mode == 4)
    {
      dest[i] = index == EMPTY_SLOT ? EMPTY_SLOT : index + row_offset;
      continue;
    }
    if (mode == 3)
    {
      uint32_t mapped = index == EMPTY_SLOT ? EMPTY_SLOT : source[(uint64_t)index * map_stride];
      dest[i] = mapped == EMPTY_SLOT ? EMPTY_SLOT : mapped + map_offset;
      continue;
    }
    bool has = index != EMPTY_SLOT;
    uint64_t row = (uint64_t)index + row_offset;
    if (mode == 0)
    {
      uint2 v = has ? *(const uint2*)(source + row * 2) : make_uint2(0, 0);
      *(uint2*)(dest + i * 2) = v;
    }
    else dest[i] = has ? source[row] : 0u;
  }
}

static int launch_selection_gather(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t count = cql_word(a, 0);
  if (count == 0) return 0;
  k_selection_gather<<<cql_stream_grid((count + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, count);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// Row materialization: the values of the selected rows of many columns, the multi-column form of the
// reference's per-column gathers (selection_gather.comp modes 0 and 1, qe_selection_gather_column
// query_exec.c:4371-4410). One launch covers up to GATHER_COLUMNS columns, column j on blockIdx.y,
// so the selected row numbers are read once per column from L2 and every store is coalesced.
//
//  cql_gather_columns  binding 0 selected rows (u32), 1 per-column params (u32 x 4: kind, base,
//                      destination byte offset lo, hi), 2 destination, 3.. the columns' buffers;
//                      word 0 count, word 2 1 = rows given (else rows 0..count-1), word 4 columns.
//                      kind 0 4-byte values, 1 u8 codes (base + code), 2 u16 codes, 3 a sequence
//                      (base + row, nothing read), 4 8-byte values, 5 1-byte values (BOOL)
//  cql_gather_string_lengths  binding 0 rows, 1 the column's (rows + 1) u64 offsets, 2 lengths (u32);
//                      word 0 count, word 2 rows given
//  cql_gather_string_bytes    binding 0 rows, 1 offsets (u64), 2 the column's bytes, 3 output offsets
//                      (u32, the exclusive scan of the lengths), 4 output bytes; word 0 count, word 2
//                      rows given. A warp per selected row, its lanes over the row's bytes.
// A row past a column's buffer reads as zero (the host checks the selection first).

#define GATHER_COLUMNS 13

__global__ void __launch_bounds__(HASH_THREADS) k_gather_columns(CqlLaunch a, uint64_t count)
{
  const uint32_t* rows = (const uint32_t*)a.buf[0];
  const uint32_t* params = (const uint32_t*)a.buf[1];
  unsigned char* dest = (unsigned char*)a.buf[2];
  bool given = cql_word(a, 2) != 0;
  uint32_t j = blockIdx.y;
  const uint32_t* pj = params + j * 4;
  uint32_t kind = pj[0], base = pj[1];
  uint64_t off = (uint64_t)pj[2] | ((uint64_t)pj[3] << 32);
  const void* src = a.buf[3 + j];
  uint64_t src_bytes = a.bytes[3 + j];
  // the column's section must lie inside the destination
  uint64_t size = kind == 4 ? 8 : kind == 5 ? 1 : 4;
  if (off % size != 0 || off > a.bytes[2] || count > (a.bytes[2] - off) / size) return;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint64_t r = given ? rows[i] : i;
    switch (kind)
    {
      case 0: ((uint32_t*)(dest + off))[i] = (r + 1) * 4 <= src_bytes ? ((const uint32_t*)src)[r] : 0u; break;
      case 1: ((uint32_t*)(dest + off))[i] = base + (r < src_bytes ? (uint32_t)((const uint8_t*)src)[r] : 0u); break;
      case 2: ((uint32_t*)(dest + off))[i] = base + ((r + 1) * 2 <= src_bytes ? (uint32_t)((const uint16_t*)src)[r] : 0u); break;
      case 3: ((uint32_t*)(dest + off))[i] = base + (uint32_t)r; break;
      case 4: ((unsigned long long*)(dest + off))[i] = (r + 1) * 8 <= src_bytes ? ((const unsigned long long*)src)[r] : 0ull; break;
      default: (dest + off)[i] = r < src_bytes ? ((const uint8_t*)src)[r] : (uint8_t)0; break;
    }
  }
}

__global__ void __launch_bounds__(HASH_THREADS) k_gather_string_lengths(CqlLaunch a, uint64_t count)
{
  const uint32_t* rows = (const uint32_t*)a.buf[0];
  const unsigned long long* offsets = (const unsigned long long*)a.buf[1];
  uint32_t* lengths = (uint32_t*)a.buf[2];
  bool given = cql_word(a, 2) != 0;
  uint64_t n_off = a.bytes[1] / 8;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint64_t r = given ? rows[i] : i;
    lengths[i] = r + 1 < n_off ? (uint32_t)(offsets[r + 1] - offsets[r]) : 0u;
  }
}

__global__ void __launch_bounds__(HASH_THREADS) k_gather_string_bytes(CqlLaunch a, uint64_t count)
{
  const uint32_t* rows = (const uint32_t*)a.buf[0];
  const unsigned long long* offsets = (const unsigned long long*)a.buf[1];
  const unsigned char* bytes = (const unsigned char*)a.buf[2];
  const uint32_t* out_off = (const uint32_t*)a.buf[3];
  unsigned char* out = (unsigned char*)a.buf[4];
  bool given = cql_word(a, 2) != 0;
  uint64_t n_off = a.bytes[1] / 8, n_bytes = a.bytes[2], out_cap = a.bytes[4];
  uint32_t lane = threadIdx.x & 31u;
  uint64_t warps = (uint64_t)gridDim.x * (blockDim.x / 32);
  for (uint64_t i = (uint64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); i < count; i += warps)
  {
    uint64_t r = given ? rows[i] : i;
    if (r + 1 >= n_off) continue;
    uint64_t s = offsets[r], e = offsets[r + 1], d = out_off[i];
    if (e > n_bytes || s > e || d + (e - s) > out_cap) continue;
    for (uint64_t b = lane; b < e - s; b += 32) out[d + b] = bytes[s + b];
  }
}

static int launch_gather_columns(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t count = cql_word(a, 0);
  uint32_t cols = cql_word(a, 4);
  if (count == 0 || cols == 0) return 0;
  if (cols > GATHER_COLUMNS || a.bytes[1] < cols * 16ull || (cql_word(a, 2) && a.bytes[0] < count * 4)) return (int)cudaErrorInvalidValue;
  uint32_t blocks = cql_stream_grid((count + HASH_THREADS - 1) / HASH_THREADS, 8);
  uint32_t x = (blocks + cols - 1) / cols;
  k_gather_columns<<<dim3(x ? x : 1, cols), HASH_THREADS, 0, stream>>>(a, count);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_gather_string_lengths(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t count = cql_word(a, 0);
  if (count == 0) return 0;
  if (a.bytes[2] < count * 4 || (cql_word(a, 2) && a.bytes[0] < count * 4)) return (int)cudaErrorInvalidValue;
  k_gather_string_lengths<<<cql_stream_grid((count + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, count);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_gather_string_bytes(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t count = cql_word(a, 0);
  if (count == 0) return 0;
  if (a.bytes[3] < count * 4 || (cql_word(a, 2) && a.bytes[0] < count * 4)) return (int)cudaErrorInvalidValue;
  uint32_t warps = HASH_THREADS / 32;
  k_gather_string_bytes<<<cql_stream_grid((count + warps - 1) / warps, 8), HASH_THREADS, 0, stream>>>(a, count);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// cql_group_finish: the hash group-by's per-group outputs in the caller's layout, on the device: binding
// 0 the compacted owner row per group (u32), 1 the row count per group (u32), 2 representative rows out
// (u64), 3 counts out (u64); with word 8 set also the results of the fixed-point reduce: binding 4 sums
// (i64 [group][expr]), 5 mins, 6 maxs (i32), 7 results out (f64 [group][expr]). Words 0 groups, 2 exprs,
// 4 funcs (4 bits each), 6 the power-of-ten exponents (4 bits each), 8 results wanted. A scaled integer
// becomes its value as the host finalized it (query_exec.c:11750-11773): the double of the integer
// divided by 10^s, AVG divided by the count after that.

__constant__ double c_pow10[7] = { 1.0, 10.0, 100.0, 1000.0, 10000.0, 100000.0, 1000000.0 };

__global__ void __launch_bounds__(HASH_THREADS) k_group_finish(CqlLaunch a, uint64_t groups)
{
  const uint32_t* owner = (const uint32_t*)a.buf[0];
  const uint32_t* count = (const uint32_t*)a.buf[1];
  unsigned long long* repr = (unsigned long long*)a.buf[2];
  unsigned long long* counts = (unsigned long long*)a.buf[3];
  const long long* sums = (const long long*)a.buf[4];
  const int* mins = (const int*)a.buf[5];
  const int* maxs = (const int*)a.buf[6];
  double* results = (double*)a.buf[7];
  uint32_t exprs = min(cql_word(a, 2), 8u), funcs = cql_word(a, 4), scales = cql_word(a, 6);
  bool finish = cql_word(a, 8) != 0;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < groups; g += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t c = count[g];
    repr[g] = owner[g];
    counts[g] = c;
    if (!finish) continue;
    for (uint32_t e = 0; e < exprs; e++)
    {
      uint64_t i = g * exprs + e;
      uint32_t f = (funcs >> (4 * e)) & 0xfu;
      double divisor = c_pow10[min((scales >> (4 * e)) & 0xfu, 6u)];
      double n = (double)c, r;
      switch (f)
      {
        case FUNC_COUNT: r = n; break;
        case FUNC_SUM: r = (double)sums[i] / divisor; break;
        case FUNC_AVG: r = c > 0 ? (double)sums[i] / divisor / n : 0.0; break;
        case FUNC_MIN: r = (double)mins[i] / divisor; break;
        default: r = (double)maxs[i] / divisor; break;
      }
      results[i] = r;
    }
  }
}

static int launch_group_finish(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t groups = cql_word(a, 0);
  if (groups == 0) return 0;
  uint64_t cells = groups * min(cql_word(a, 2), 8u);
  if (a.bytes[0] < groups * 4 || a.bytes[1] < groups * 4 || a.bytes[2] < groups * 8 || a.bytes[3] < groups * 8)
    return (int)cudaErrorInvalidValue;
  if (cql_word(a, 8) && (a.bytes[4] < cells * 8 || a.bytes[5] < cells * 4 || a.bytes[6] < cells * 4 || a.bytes[7] < cells * 8))
    return (int)cudaErrorInvalidValue;
  k_group_finish<<<cql_stream_grid((groups + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, groups);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// cql_group_small: GROUP BY a small-range whole-number key (at most 64 values) in one pass over the key
// and up to 8 argument columns: per value of the key its row count, first row, and per column the exact
// SUM and the MIN and MAX.
//
// A SUM is exact in fixed point: each value x of a column becomes the whole number q = round(x * 2^s),
// with s chosen from the column's range so that |q| < 2^61 (s = 0 for whole-number columns, which are then
// exact), and the q are added as 96-bit two's-complement numbers (a thread's own table: a u64 low part and
// a u32 high part; tables shared by threads: three 32-bit limbs, shared atomics with the carries passed up,
// as the dense group-by's 64-bit sums do), then as 128-bit numbers in the output. The host turns the total back into a double, rounding once: the f64 SUM is the exact sum of the
// values rounded to 2^-s, whose error is below rows * 2^(E-62) for values below 2^E - far inside the
// 1e-12 the sum is held to, and independent of the order the rows are met in. NaN and infinite values are
// kept out of the sum and flagged (NaN 1, +inf 2, -inf 4), so that the host gives the IEEE result.
//
// binding 0 the key (u32 words), 1..8 the argument columns, 9 the output (u32 words, for V key values):
//   [0, 2V)           the counts (u64)
//   [2V, 3V)          the first rows (u32; all 0xffffffff before)
//   S = 3V + (V & 1)  per (value, column) 4 words: the sum as a 128-bit two's-complement number
//   S + 32V           per (value, column) the flags
//   S + 40V           per (value, column) the (min, max) as f64 order keys (u64 pairs; min all ones and max
//                     zero before)
// words: 0 rows, 2 the smallest key (bits), 4 V, 6 the columns, 8 their CQL types (4 bits each: U32, I32,
// F32, F64), 10 per column 1 = SUM (bits 0-7) and 1 = MIN/MAX (bits 8-15), slots 6 and 7 the columns'
// scales s (signed 16 bits each, columns 0-3 then 4-7). Dynamic shared memory: `copies` private tables of
// V counts and one sum per summed column and value (laid out below the kernel's head); with one table a
// thread (OWN) they are updated without atomics.

#define SMALL_VALUES 64
#define SMALL_COLUMNS 8
#define SMALL_ROWS 4

// The per-row work is integer work on the values' IEEE bits (GB300's FP64 pipe is a small fraction of its
// integer and FP32 rate): a value becomes the bits of its double, then a fixed-point whole number or an
// order key.

// the double bits of a 32-bit float (exact: subnormals normalized, infinities and NaN kept)
__device__ __forceinline__ unsigned long long small_f32_bits(uint32_t b)
{
  unsigned long long sign = (unsigned long long)(b >> 31) << 63;
  uint32_t e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  if (e == 0xffu) return sign | 0x7ff0000000000000ull | ((unsigned long long)m << 29);
  if (e == 0)
  {
    if (m == 0) return sign;
    uint32_t shift = __clz(m) - 8;   // bring the leading one to bit 23
    m = (m << shift) & 0x7fffffu;
    return sign | ((unsigned long long)(1023 - 126 - shift) << 52) | ((unsigned long long)m << 29);
  }
  return sign | ((unsigned long long)(e - 127 + 1023) << 52) | ((unsigned long long)m << 29);
}

// the double bits of a whole number below 2^53 in magnitude (exact)
__device__ __forceinline__ unsigned long long small_int_bits(long long v)
{
  if (v == 0) return 0;
  unsigned long long sign = v < 0 ? 0x8000000000000000ull : 0ull, a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  int p = 63 - __clzll(a);
  return sign | ((unsigned long long)(1023 + p) << 52) | ((a << (52 - p)) & 0xfffffffffffffull);
}

// x * 2^s rounded to the nearest whole number (ties away from zero), for a finite double x given by its
// bits; |x * 2^s| < 2^62 by the choice of s
__device__ __forceinline__ long long small_fixed(unsigned long long b, int s)
{
  int e = (int)((b >> 52) & 0x7ffu);
  unsigned long long m = b & 0xfffffffffffffull;
  if (e) m |= 1ull << 52;
  else e = 1;
  int sh = e - 1075 + s;   // x * 2^s = m * 2^sh
  unsigned long long q;
  if (sh >= 0) q = sh > 10 ? (1ull << 62) : m << sh;   // past 2^62 only for a value outside the column's range
  else
  {
    // to nearest, ties away from zero: add half a unit of the last place kept, then shift (0 from 54 places down)
    uint32_t r = (uint32_t)min(-sh, 63);
    q = (m + (1ull << (r - 1))) >> r;
  }
  return (b >> 63) ? -(long long)q : (long long)q;
}

// Adds a 64-bit signed q into a 96-bit two's-complement number held as three 32-bit limbs shared by
// several threads: shared atomics, each carry passed up once.
__device__ __forceinline__ void add96_atomic(uint32_t* l0, uint32_t* l1, uint32_t* l2, long long q)
{
  uint32_t lo = (uint32_t)q, hi = (uint32_t)((unsigned long long)q >> 32), top = q < 0 ? 0xffffffffu : 0u;
  uint32_t old0 = atomicAdd(l0, lo);
  uint32_t mid = hi + ((old0 + lo < old0) ? 1u : 0u);
  top += mid < hi ? 1u : 0u;   // hi + carry passed 2^32
  if (mid)
  {
    uint32_t old1 = atomicAdd(l1, mid);
    top += (old1 + mid < old1) ? 1u : 0u;
  }
  if (top) atomicAdd(l2, top);
}

// The tables in dynamic shared memory, word-major (word w of table k at w * copies + k), so that the lanes
// of a warp, each on its own table, meet no bank conflict. With a table a thread (OWN) a sum is a u64
// low part and a u32 high part, updated without atomics; with tables shared by threads, three u32 limbs
// updated with atomics.
template <bool OWN>
__global__ void __launch_bounds__(HASH_THREADS) k_group_small(CqlLaunch a, uint64_t rows, uint32_t copies)
{
  extern __shared__ __align__(16) uint32_t smem[];
  // extrema [column][min | max][value] and flags [column][value]: a warp's lanes on different key values
  // meet different banks
  __shared__ unsigned long long s_ext[SMALL_COLUMNS * 2 * SMALL_VALUES];
  __shared__ uint32_t s_first[SMALL_VALUES], s_flags[SMALL_COLUMNS * SMALL_VALUES];
  // per column: type, sum slot, scale and what is kept (1 SUM, 2 MIN/MAX, 4 a whole-number column)
  __shared__ uint32_t s_type[SMALL_COLUMNS], s_slot[SMALL_COLUMNS], s_what[SMALL_COLUMNS];
  __shared__ int s_scale[SMALL_COLUMNS];
  const uint32_t* key = (const uint32_t*)a.buf[0];
  uint32_t* out = (uint32_t*)a.buf[1 + SMALL_COLUMNS];
  uint32_t min_key = cql_word(a, 2), V = cql_word(a, 4), ncols = cql_word(a, 6), types = cql_word(a, 8), need = cql_word(a, 10);
  uint32_t nsum = 0;
  for (uint32_t c = 0; c < ncols; c++) nsum += (need >> c) & 1u;
  if (threadIdx.x < SMALL_COLUMNS)
  {
    uint32_t c = threadIdx.x, t = (types >> (4 * c)) & 0xfu;
    s_type[c] = t;
    s_slot[c] = __popc(need & ((1u << c) - 1u) & 0xffu);
    s_what[c] = c < ncols ? (((need >> c) & 1u) | (((need >> (SMALL_COLUMNS + c)) & 1u) << 1) | ((t == 1 || t == 7) ? 4u : 0u)) : 0u;
    s_scale[c] = (int)(short)(unsigned short)(a.push[6 + c / 4] >> (16 * (c % 4)));
  }
  // counts [V][copies] (u32); OWN: sum lows [nsum][V][copies] (u64) then highs (u32); else limbs
  // [nsum][3][V][copies] (u32) (copies is a power of two of at least 8, so the u64 lows start 8-byte aligned)
  uint32_t* cnt = smem;
  unsigned long long* sum_lo = (unsigned long long*)(smem + V * copies);
  uint32_t* sum_hi = (uint32_t*)(sum_lo + nsum * V * copies);
  uint32_t* limbs = smem + V * copies;
  uint32_t total_words = V * copies * (1 + 3 * nsum);
  for (uint32_t i = threadIdx.x; i < total_words; i += blockDim.x) smem[i] = 0;
  for (uint32_t i = threadIdx.x; i < SMALL_COLUMNS * 2 * SMALL_VALUES; i += blockDim.x)
    s_ext[i] = ((i / SMALL_VALUES) & 1u) ? 0ull : ~0ull;
  for (uint32_t i = threadIdx.x; i < SMALL_VALUES; i += blockDim.x) s_first[i] = 0xffffffffu;
  for (uint32_t i = threadIdx.x; i < SMALL_COLUMNS * SMALL_VALUES; i += blockDim.x) s_flags[i] = 0;
  __syncthreads();
  uint32_t copy = threadIdx.x % copies;
  // SMALL_ROWS rows a thread a step, a grid stride apart (each coalesced across the warp): the keys read
  // together, then each column's values together, so that a thread keeps several loads in flight
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t r0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r0 < rows; r0 += step * SMALL_ROWS)
  {
    uint32_t g[SMALL_ROWS];
#pragma unroll
    for (uint32_t i = 0; i < SMALL_ROWS; i++)
    {
      uint64_t r = r0 + i * step;
      g[i] = r < rows ? key[r] - min_key : 0xffffffffu;
    }
#pragma unroll
    for (uint32_t i = 0; i < SMALL_ROWS; i++)
    {
      if (g[i] >= V) continue;
      uint32_t r = (uint32_t)(r0 + i * step);
      if (OWN) cnt[g[i] * copies + copy] += 1;
      else atomicAdd(&cnt[g[i] * copies + copy], 1u);
      if (r < s_first[g[i]]) atomicMin(&s_first[g[i]], r);
    }
#pragma unroll 1
    for (uint32_t c = 0; c < ncols; c++)
    {
      uint32_t type = s_type[c], what = s_what[c], slot = s_slot[c];
      int scale = s_scale[c];
      bool whole_col = (what & 4u) != 0;
      const void* col = a.buf[1 + c];
      unsigned long long raw[SMALL_ROWS];
#pragma unroll
      for (uint32_t i = 0; i < SMALL_ROWS; i++)
      {
        uint64_t r = r0 + i * step;
        raw[i] = 0;
        if (r < rows) raw[i] = type == 4 ? ((const unsigned long long*)col)[r] : ((const uint32_t*)col)[r];
      }
#pragma unroll
      for (uint32_t i = 0; i < SMALL_ROWS; i++)
      {
        if (g[i] >= V) continue;
        // the value as a whole number (whole-number columns, exact) and, where needed, as its double's bits
        long long whole = type == 7 ? (long long)(int)(uint32_t)raw[i] : (long long)raw[i];
        unsigned long long b = 0;
        if (!whole_col) b = type == 3 ? small_f32_bits((uint32_t)raw[i]) : raw[i];
        bool finite = whole_col || ((b >> 52) & 0x7ffu) != 0x7ffu;
        if (what & 1u)
        {
          if (finite)
          {
            long long q = whole_col ? whole : small_fixed(b, scale);
            if (OWN)
            {
              uint32_t at = (slot * V + g[i]) * copies + copy;
              unsigned long long old = sum_lo[at], now = old + (unsigned long long)q;
              sum_lo[at] = now;
              uint32_t top = (q < 0 ? 0xffffffffu : 0u) + (now < old ? 1u : 0u);
              if (top) sum_hi[at] += top;
            }
            else
            {
              uint32_t at3 = ((slot * 3) * V + g[i]) * copies + copy, stride = V * copies;
              add96_atomic(limbs + at3, limbs + at3 + stride, limbs + at3 + 2 * stride, q);
            }
          }
          else
            atomicOr(&s_flags[c * SMALL_VALUES + g[i]], (b & 0xfffffffffffffull) ? 1u : (b >> 63) ? 4u : 2u);
        }
        if (what & 2u)
        {
          if (whole_col) b = small_int_bits(whole);
          if (finite || !(b & 0xfffffffffffffull))   // NaN is left out
          {
            if ((b << 1) == 0) b = 0;   // -0.0 compares equal to +0.0
            unsigned long long o = (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
            unsigned long long* e = s_ext + c * 2 * SMALL_VALUES + g[i];
            if (o < e[0]) atomicMin(&e[0], o);
            if (o > e[SMALL_VALUES]) atomicMax(&e[SMALL_VALUES], o);
          }
        }
      }
    }
  }
  __syncthreads();
  // this CTA's tables folded and added to the output: counts (u64), sums (128-bit), first rows, extrema, flags
  unsigned long long* counts = (unsigned long long*)out;
  uint32_t sums_at = 3 * V + (V & 1u);
  unsigned long long* sums = (unsigned long long*)(out + sums_at);
  uint32_t* flags = out + sums_at + 4 * SMALL_COLUMNS * V;
  unsigned long long* ext = (unsigned long long*)(out + sums_at + 5 * SMALL_COLUMNS * V);
  for (uint32_t t = threadIdx.x; t < V * (1 + nsum); t += blockDim.x)
  {
    uint32_t g = t % V, part = t / V;
    if (part == 0)
    {
      unsigned long long n = 0;
      for (uint32_t k = 0; k < copies; k++) n += cnt[g * copies + k];
      if (n) atomicAdd(&counts[g], n);
      continue;
    }
    uint32_t slot = part - 1;
    __int128 total = 0;
    for (uint32_t k = 0; k < copies; k++)
    {
      if (OWN)
      {
        uint32_t at = (slot * V + g) * copies + k;
        total += (__int128)(((unsigned __int128)(unsigned long long)(long long)(int)sum_hi[at] << 64) | sum_lo[at]);
      }
      else
      {
        uint32_t at3 = ((slot * 3) * V + g) * copies + k, stride = V * copies;
        unsigned long long low = (unsigned long long)limbs[at3] | ((unsigned long long)limbs[at3 + stride] << 32);
        total += (__int128)(((unsigned __int128)(unsigned long long)(long long)(int)limbs[at3 + 2 * stride] << 64) | low);
      }
    }
    if (total == 0) continue;
    // the summed column whose slot this is
    uint32_t c = 0;
    for (uint32_t j = 0; j < ncols; j++)
      if ((s_what[j] & 1u) && s_slot[j] == slot) c = j;
    unsigned long long lo = (unsigned long long)total, hi = (unsigned long long)((unsigned __int128)total >> 64);
    unsigned long long* at = sums + (g * SMALL_COLUMNS + c) * 2;
    unsigned long long old = atomicAdd(&at[0], lo);
    hi += (old + lo < old) ? 1ull : 0ull;
    if (hi) atomicAdd(&at[1], hi);
  }
  for (uint32_t t = threadIdx.x; t < V * SMALL_COLUMNS; t += blockDim.x)
  {
    // t = g * SMALL_COLUMNS + c in the output's order
    uint32_t g = t / SMALL_COLUMNS, c = t % SMALL_COLUMNS;
    if (c == 0 && s_first[g] != 0xffffffffu) atomicMin(&out[2 * V + g], s_first[g]);
    uint32_t f = s_flags[c * SMALL_VALUES + g];
    if (f) atomicOr(&flags[t], f);
    unsigned long long lo = s_ext[c * 2 * SMALL_VALUES + g], hi = s_ext[c * 2 * SMALL_VALUES + SMALL_VALUES + g];
    if (lo != ~0ull) atomicMin(&ext[2 * t], lo);
    if (hi != 0ull) atomicMax(&ext[2 * t + 1], hi);
  }
}

// cql_group_direct: GROUP BY one whole-number key of a dense range too large for shared memory (R values
// from the smallest, R <= 2^24) over whole-number arguments, straight into tables in device memory indexed
// by key - min (a few MB: they stay in L2), with atomics whose results are not read. Binding 0 the key (u32
// words), 1..8 the argument columns (u32/i32 words, values inside the i32 range), 9 the tables (u32
// words): counts [R] at 0, first rows [R] at R (all 0xffffffff before), then expression e's table at word
// offset slot 4 + e/2 (half e%2): SUM/AVG an i64 [R] (8-byte aligned), MIN/MAX an i32 [R] (INT32_MAX /
// INT32_MIN before). Words: 0 rows, 2 the smallest key (bits), 3 R, 4 expressions, 5 their functions (4
// bits each), 6 per expression 1 = an I32 argument.
#define DIRECT_ROWS 4

__global__ void __launch_bounds__(HASH_THREADS) k_group_direct(CqlLaunch a, uint64_t rows)
{
  const uint32_t* key = (const uint32_t*)a.buf[0];
  uint32_t* tab = (uint32_t*)a.buf[9];
  uint32_t kmin = cql_word(a, 2), R = cql_word(a, 3), exprs = min(cql_word(a, 4), 8u), funcs = cql_word(a, 5), sgn = cql_word(a, 6);
  uint32_t* cnt = tab;
  uint32_t* first = tab + R;
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t r0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r0 < rows; r0 += step * DIRECT_ROWS)
  {
    uint32_t k[DIRECT_ROWS];
#pragma unroll
    for (uint32_t i = 0; i < DIRECT_ROWS; i++)
    {
      uint64_t r = r0 + i * step;
      k[i] = r < rows ? key[r] - kmin : 0xffffffffu;
    }
#pragma unroll
    for (uint32_t i = 0; i < DIRECT_ROWS; i++)
    {
      if (k[i] >= R) continue;
      // atomics whose results are not read: the L2 performs them, the thread does not wait (a read of the
      // first row before its atomic would cost the same L2 operation plus the wait)
      atomicAdd(&cnt[k[i]], 1u);
      atomicMin(&first[k[i]], (uint32_t)(r0 + i * step));
    }
#pragma unroll 1
    for (uint32_t e = 0; e < exprs; e++)
    {
      uint32_t f = (funcs >> (4 * e)) & 0xfu;
      if (f == FUNC_COUNT) continue;
      const uint32_t* col = (const uint32_t*)a.buf[1 + e];
      bool is_signed = (sgn >> e) & 1u;
      uint32_t off = cql_word(a, 8 + e);
      uint32_t v[DIRECT_ROWS];
#pragma unroll
      for (uint32_t i = 0; i < DIRECT_ROWS; i++)
      {
        uint64_t r = r0 + i * step;
        v[i] = (r < rows && k[i] < R) ? col[r] : 0u;
      }
#pragma unroll
      for (uint32_t i = 0; i < DIRECT_ROWS; i++)
      {
        if (k[i] >= R) continue;
        if (f == FUNC_SUM || f == FUNC_AVG)
        {
          long long x = is_signed ? (long long)(int)v[i] : (long long)v[i];
          atomicAdd((unsigned long long*)(tab + off) + k[i], (unsigned long long)x);
        }
        else if (f == FUNC_MIN)
          atomicMin((int*)(tab + off) + k[i], (int)v[i]);
        else
          atomicMax((int*)(tab + off) + k[i], (int)v[i]);
      }
    }
  }
}

// cql_group_direct_bits: binding 0 the counts [R], 1 a bitmap of the present keys out (bit k = count > 0),
// 2 the number of present keys (u32, zero before); word 0 R.
__global__ void __launch_bounds__(HASH_THREADS) k_group_direct_bits(CqlLaunch a, uint32_t R)
{
  __shared__ uint32_t s_present;
  const uint32_t* cnt = (const uint32_t*)a.buf[0];
  uint32_t* bits = (uint32_t*)a.buf[1];
  uint32_t* present = (uint32_t*)a.buf[2];
  uint32_t words = (R + 31) / 32, mine = 0;
  if (threadIdx.x == 0) s_present = 0;
  __syncthreads();
  for (uint64_t w0 = (uint64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x / 32); w0 < words; w0 += (uint64_t)gridDim.x * (blockDim.x / 32))
  {
    uint64_t k = w0 * 32 + (threadIdx.x & 31);
    uint32_t m = __ballot_sync(0xffffffffu, k < R && cnt[k] != 0);
    if ((threadIdx.x & 31) == 0)
    {
      bits[w0] = m;
      mine += (uint32_t)__popc(m);
    }
  }
  // one atomic a CTA on the shared count (a global atomic a warp word would all meet on one address)
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(&s_present, mine);
  __syncthreads();
  if (threadIdx.x == 0 && s_present) atomicAdd(present, s_present);
}

// cql_group_direct_emit: the groups in key order in the caller's layout: binding 0 the tables, 1 the present
// keys (ascending offsets from the smallest key), 2 the number of them, 3 representative (first) rows out
// (u64), 4 counts out (u64), 5 results out (f64 [group][expr]); words as cql_group_direct's (0 rows unused,
// 3 R, 4 expressions, 5 functions, 8.. the table offsets). The results are those of the fixed-point
// reduce at scale 0: the double of the sum, AVG that divided by the count, MIN/MAX the double of the value.
__global__ void __launch_bounds__(HASH_THREADS) k_group_direct_emit(CqlLaunch a, uint64_t cap)
{
  const uint32_t* tab = (const uint32_t*)a.buf[0];
  const uint32_t* list = (const uint32_t*)a.buf[1];
  uint32_t groups = *(const uint32_t*)a.buf[2];
  unsigned long long* repr = (unsigned long long*)a.buf[3];
  unsigned long long* counts = (unsigned long long*)a.buf[4];
  double* results = (double*)a.buf[5];
  uint32_t R = cql_word(a, 3), exprs = min(cql_word(a, 4), 8u), funcs = cql_word(a, 5);
  uint64_t n = min((uint64_t)groups, cap);
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t k = list[g];
    if (k >= R) continue;
    uint32_t c = tab[k];
    repr[g] = tab[R + k];
    counts[g] = c;
    for (uint32_t e = 0; e < exprs; e++)
    {
      uint32_t f = (funcs >> (4 * e)) & 0xfu, off = cql_word(a, 8 + e);
      double r;
      if (f == FUNC_COUNT) r = (double)c;
      else if (f == FUNC_SUM || f == FUNC_AVG)
      {
        double sum = (double)((const long long*)(tab + off))[k];
        r = f == FUNC_AVG ? (c > 0 ? sum / (double)c : 0.0) : sum;
      }
      else r = (double)((const int*)(tab + off))[k];
      results[g * exprs + e] = r;
    }
  }
}

static int launch_group_direct(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = a.push[0];
  uint32_t R = cql_word(a, 3), exprs = cql_word(a, 4), funcs = cql_word(a, 5);
  if (rows == 0) return 0;
  if (R == 0 || R > (1u << 24) || exprs == 0 || exprs > 8 || rows > 0xffffffffull || a.bytes[0] < rows * 4) return (int)cudaErrorInvalidValue;
  uint64_t words = a.bytes[9] / 4;
  if (words < 2ull * R) return (int)cudaErrorInvalidValue;
  for (uint32_t e = 0; e < exprs; e++)
  {
    uint32_t f = (funcs >> (4 * e)) & 0xfu;
    if (f == FUNC_COUNT) continue;
    if (f > FUNC_MAX || a.bytes[1 + e] < rows * 4) return (int)cudaErrorInvalidValue;
    uint64_t off = cql_word(a, 8 + e), need = (f == FUNC_SUM || f == FUNC_AVG) ? 2ull * R : R;
    if (off < 2ull * R || off + need > words || ((f == FUNC_SUM || f == FUNC_AVG) && (off & 1))) return (int)cudaErrorInvalidValue;
  }
  k_group_direct<<<cql_stream_grid((rows + HASH_THREADS * DIRECT_ROWS - 1) / (HASH_THREADS * DIRECT_ROWS), 8), HASH_THREADS, 0, stream>>>(a, rows);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_group_direct_bits(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint32_t R = cql_word(a, 0);
  if (R == 0) return 0;
  if (a.bytes[0] < (uint64_t)R * 4 || a.bytes[1] < (uint64_t)((R + 31) / 32) * 4 || a.bytes[2] < 4) return (int)cudaErrorInvalidValue;
  uint64_t warps = (R + 31) / 32;
  k_group_direct_bits<<<cql_stream_grid((warps + HASH_THREADS / 32 - 1) / (HASH_THREADS / 32), 8), HASH_THREADS, 0, stream>>>(a, R);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_group_direct_emit(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint32_t R = cql_word(a, 3), exprs = cql_word(a, 4), funcs = cql_word(a, 5);
  if (R == 0 || exprs == 0 || exprs > 8 || a.bytes[2] < 4) return (int)cudaErrorInvalidValue;
  uint64_t words = a.bytes[0] / 4;
  if (words < 2ull * R) return (int)cudaErrorInvalidValue;
  for (uint32_t e = 0; e < exprs; e++)
  {
    uint32_t f = (funcs >> (4 * e)) & 0xfu;
    if (f == FUNC_COUNT) continue;
    uint64_t off = cql_word(a, 8 + e), need = (f == FUNC_SUM || f == FUNC_AVG) ? 2ull * R : R;
    if (f > FUNC_MAX || off + need > words) return (int)cudaErrorInvalidValue;
  }
  // the most groups each output holds
  uint64_t cap = a.bytes[1] / 4;
  cap = std::min<uint64_t>(cap, a.bytes[3] / 8);
  cap = std::min<uint64_t>(cap, a.bytes[4] / 8);
  cap = std::min<uint64_t>(cap, a.bytes[5] / (8ull * exprs));
  if (cap == 0) return 0;
  uint64_t most = std::min<uint64_t>(cap, R);
  k_group_direct_emit<<<cql_stream_grid((most + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, cap);
  CQL_LAUNCH_CHECK();
  return 0;
}

// cql_finite_magnitude: the largest finite |x| of an f32/f64 column, as the bits of a non-negative double
// (whose order is the bits' order): binding 0 the column, 1 the result (u64, zero before); word 0 rows,
// word 2 the CQL type (F32 or F64). The small-key GROUP BY's scale for a column with no finite range.
__global__ void __launch_bounds__(HASH_THREADS) k_finite_magnitude(CqlLaunch a, uint64_t rows, bool f32)
{
  unsigned long long best = 0;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (uint64_t)gridDim.x * blockDim.x)
  {
    double x = f32 ? (double)((const float*)a.buf[0])[r] : ((const double*)a.buf[0])[r];
    if (isfinite(x)) best = max(best, (unsigned long long)__double_as_longlong(fabs(x)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
  __shared__ unsigned long long s_best;
  if (threadIdx.x == 0) s_best = 0;
  __syncthreads();
  if ((threadIdx.x & 31u) == 0 && best) atomicMax(&s_best, best);
  __syncthreads();
  if (threadIdx.x == 0 && s_best) atomicMax((unsigned long long*)a.buf[1], s_best);
}

static int launch_finite_magnitude(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = a.push[0];
  uint32_t type = cql_word(a, 2);
  if (rows == 0) return 0;
  if (!(type == 3 || type == 4) || a.bytes[0] < rows * (type == 4 ? 8 : 4) || a.bytes[1] < 8) return (int)cudaErrorInvalidValue;
  k_finite_magnitude<<<cql_stream_grid((rows + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, rows, type == 3);
  CQL_LAUNCH_CHECK();
  return 0;
}

// the output's size in u32 words for V key values
static uint64_t group_small_words(uint32_t V)
{
  return 3ull * V + (V & 1u) + 9ull * SMALL_COLUMNS * V;
}

static int launch_group_small(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = a.push[0];
  if (rows == 0) return 0;
  uint32_t V = cql_word(a, 4), ncols = cql_word(a, 6), types = cql_word(a, 8), need = cql_word(a, 10);
  if (V == 0 || V > SMALL_VALUES || ncols > SMALL_COLUMNS || rows > 0xffffffffull || a.bytes[0] < rows * 4 ||
      a.bytes[1 + SMALL_COLUMNS] < group_small_words(V) * 4)
    return (int)cudaErrorInvalidValue;
  uint32_t nsum = 0;
  for (uint32_t c = 0; c < ncols; c++)
  {
    uint32_t t = (types >> (4 * c)) & 0xfu;
    uint64_t width = t == 4 ? 8 : 4;
    if (!(t == 1 || t == 7 || t == 3 || t == 4) || a.bytes[1 + c] < rows * width) return (int)cudaErrorInvalidValue;
    nsum += (need >> c) & 1u;
  }
  // private tables: one a thread when they fit in 48 KB, else as many as fit (a power of two, at least one a warp)
  uint32_t table_bytes = V * (1 + 3 * nsum) * 4;
  uint32_t copies = HASH_THREADS;
  while (copies > 8 && (uint64_t)copies * table_bytes > 48u * 1024u) copies >>= 1;
  size_t smem = (size_t)copies * table_bytes;
  bool own = copies == HASH_THREADS;
  const void* fn = own ? (const void*)k_group_small<true> : (const void*)k_group_small<false>;
  // with the static tables (extrema, flags, first rows) the CTA passes the default 48 KB: opt in
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, HASH_THREADS, smem) != cudaSuccess || per_sm < 1)
  {
    cudaGetLastError();
    per_sm = 1;
  }
  uint32_t grid = cql_stream_grid((rows + HASH_THREADS - 1) / HASH_THREADS, per_sm);
  if (own) k_group_small<true><<<grid, HASH_THREADS, smem, stream>>>(a, rows, copies);
  else k_group_small<false><<<grid, HASH_THREADS, smem, stream>>>(a, rows, copies);
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// Widening of a device column to dense f64 (the gather the operator layer does on the host before
// a hash GROUP BY, query_exec.c:10454-10690): binding 0 source, 1 destination; word 0 rows, word 2
// the source CQL type. Not a reference kernel: the reference uploads the f64 copy it builds on the host.

__global__ void __launch_bounds__(HASH_THREADS) k_widen_f64(CqlLaunch a, uint64_t rows, uint32_t type)
{
  const uint32_t* s = (const uint32_t*)a.buf[0];
  double* d = (double*)a.buf[1];
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (uint64_t)gridDim.x * blockDim.x)
  {
    double v;
    switch (type)
    {
      case 1: v = (double)s[i]; break;
      case 7: v = (double)(int)s[i]; break;
      case 3: v = (double)__uint_as_float(s[i]); break;
      case 4: v = ((const double*)s)[i]; break;
      case 2: v = (double)((const unsigned long long*)s)[i]; break;
      default: v = (double)((const long long*)s)[i]; break;
    }
    d[i] = v;
  }
}

static int launch_widen_f64(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t rows = a.push[0];
  if (rows == 0) return 0;
  k_widen_f64<<<cql_stream_grid((rows + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, rows, cql_word(a, 2));
  CQL_LAUNCH_CHECK();
  return 0;
}

// ---------------------------------------------------------------------------------------------
// The member-list layout of the CSR reduce, built on the device (the reference builds it on the host,
// query_exec.c:11826-11990): group starts and chunk bases are prefix sums (prefix_sum), these kernels
// fill the rest and fold each group's chunk partials in chunk order.
//
//  cql_group_chunks  binding 0 rows per group (u32), 1 chunks per group (u32 out); word 0 groups,
//                    word 2 rows per chunk. A group of no rows still has one chunk.
//  cql_slot_cursor   binding 0 rows per slot, 1 slot -> group (compact offsets), 2 group starts,
//                    3 cursor per slot (out); word 0 slots
//  cql_chunk_ranges  binding 0 group starts, 1 rows per group, 2 chunk bases, 3 chunk (first, end) row
//                    pairs (out), 4 chunk group (out); word 0 groups, word 2 rows per chunk
//  cql_group_fold    binding 0 partials (chunk, expr) x (sum, count, min, max) f64, 1 chunk bases
//                    (groups + 1), 2 results (group, expr) f64 (out); word 0 groups, 2 exprs, 4 codes

__global__ void __launch_bounds__(HASH_THREADS) k_group_chunks(CqlLaunch a, uint32_t groups, uint32_t per_chunk)
{
  const uint32_t* count = (const uint32_t*)a.buf[0];
  uint32_t* chunks = (uint32_t*)a.buf[1];
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < groups; g += gridDim.x * blockDim.x)
    chunks[g] = count[g] ? (count[g] + per_chunk - 1) / per_chunk : 1u;
}

__global__ void __launch_bounds__(HASH_THREADS) k_slot_cursor(CqlLaunch a, uint64_t slots, uint32_t groups)
{
  const uint32_t* count = (const uint32_t*)a.buf[0];
  const uint32_t* group_of = (const uint32_t*)a.buf[1];
  const uint32_t* start = (const uint32_t*)a.buf[2];
  uint32_t* cursor = (uint32_t*)a.buf[3];
  for (uint64_t sl = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; sl < slots; sl += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t g = group_of[sl];
    cursor[sl] = (count[sl] && g < groups) ? start[g] : 0u;
  }
}

// one warp per group: a group of 10M rows has ~2400 chunks
__global__ void __launch_bounds__(HASH_THREADS) k_chunk_ranges(CqlLaunch a, uint32_t groups, uint32_t per_chunk, uint64_t chunk_cap)
{
  const uint32_t* start = (const uint32_t*)a.buf[0];
  const uint32_t* count = (const uint32_t*)a.buf[1];
  const uint32_t* base = (const uint32_t*)a.buf[2];
  uint32_t* range = (uint32_t*)a.buf[3];
  uint32_t* group = (uint32_t*)a.buf[4];
  uint32_t lane = threadIdx.x & 31u;
  uint64_t warps = (uint64_t)gridDim.x * (blockDim.x / 32);
  for (uint64_t g = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; g < groups; g += warps)
  {
    uint32_t n = base[g + 1] - base[g], s = start[g], e = start[g] + count[g];
    for (uint32_t k = lane; k < n; k += 32)
    {
      uint64_t c = (uint64_t)base[g] + k;
      if (c >= chunk_cap) break;
      uint32_t first = s + k * per_chunk;
      range[c * 2] = first;
      range[c * 2 + 1] = min(first + per_chunk, e);
      group[c] = (uint32_t)g;
    }
  }
}

// The fold of each group's chunk partials, in chunk order for SUM/AVG (the same sequence of f64
// additions as the reference's host fold); COUNT, MIN and MAX do not depend on the order (counts are
// whole numbers far below 2^53). A warp takes 32 consecutive groups: a lane folds its own group when it
// has few chunks, and the warp folds the groups of many chunks together, one after the other.
__device__ __forceinline__ double fold_result(uint32_t f, double acc, double cnt, double mn, double mx)
{
  if (f == 0) return cnt;
  if (f == 1) return acc;
  if (f == 2) return cnt > 0.0 ? __ddiv_rn(acc, cnt) : 0.0;
  if (f == 3) return mn;
  if (f == 4) return mx;
  return 0.0;   // sketches are finished on the host
}

__global__ void __launch_bounds__(HASH_THREADS) k_group_fold(CqlLaunch a, uint32_t groups, uint32_t exprs, uint32_t codes)
{
  const double* partials = (const double*)a.buf[0];
  const uint32_t* base = (const uint32_t*)a.buf[1];
  double* results = (double*)a.buf[2];
  uint64_t limit = a.bytes[0] / 32 / exprs;
  uint32_t lane = threadIdx.x & 31u;
  uint64_t warps = (uint64_t)gridDim.x * (blockDim.x / 32);
  for (uint64_t g0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32 * 32; g0 < groups; g0 += warps * 32)
  {
    uint64_t g = g0 + lane;
    uint64_t first = g < groups ? base[g] : 0, end = g < groups ? min((uint64_t)base[g + 1], limit) : 0;
    bool small = end - first <= 32;
    if (g < groups && small)
      for (uint32_t e = 0; e < exprs; e++)
      {
        uint32_t f = (codes >> (4 * e)) & 0xfu;
        if (f > 4) continue;
        double acc = 0.0, mn = 1.0e300, mx = -1.0e300, cnt = 0.0;
        for (uint64_t c = first; c < end; c++)
        {
          const double* pp = &partials[(c * exprs + e) * 4];
          acc = __dadd_rn(acc, pp[0]);
          cnt = __dadd_rn(cnt, pp[1]);
          mn = pp[2] < mn ? pp[2] : mn;
          mx = pp[3] > mx ? pp[3] : mx;
        }
        results[g * exprs + e] = fold_result(f, acc, cnt, mn, mx);
      }
    uint32_t big = __ballot_sync(0xffffffffu, g < groups && !small);
    while (big)
    {
      uint32_t j = __ffs(big) - 1;
      big &= big - 1;
      uint64_t gb = g0 + j;
      uint64_t bf = __shfl_sync(0xffffffffu, first, j), be = __shfl_sync(0xffffffffu, end, j);
      for (uint32_t e = 0; e < exprs; e++)
      {
        uint32_t f = (codes >> (4 * e)) & 0xfu;
        if (f > 4) continue;
        double acc = 0.0, mn = 1.0e300, mx = -1.0e300, cnt = 0.0;
        bool ordered = f == 1 || f == 2;
        for (uint64_t c0 = bf; c0 < be; c0 += 32)
        {
          uint64_t c = c0 + lane;
          double p0 = 0.0, p1 = 0.0, p2 = 1.0e300, p3 = -1.0e300;
          if (c < be)
          {
            const double* pp = &partials[(c * exprs + e) * 4];
            p0 = pp[0];
            p1 = pp[1];
            p2 = pp[2];
            p3 = pp[3];
          }
          if (ordered)
          {
            uint32_t m = (uint32_t)min((uint64_t)32, be - c0);
            for (uint32_t k = 0; k < m; k++) acc = __dadd_rn(acc, __shfl_sync(0xffffffffu, p0, k));
          }
          // counts (whole numbers), minima and maxima: any order
          cnt = __dadd_rn(cnt, p1);
          mn = p2 < mn ? p2 : mn;
          mx = p3 > mx ? p3 : mx;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
          cnt = __dadd_rn(cnt, __shfl_xor_sync(0xffffffffu, cnt, o));
          double lo = __shfl_xor_sync(0xffffffffu, mn, o), hi = __shfl_xor_sync(0xffffffffu, mx, o);
          mn = lo < mn ? lo : mn;
          mx = hi > mx ? hi : mx;
        }
        if (lane == 0) results[gb * exprs + e] = fold_result(f, acc, cnt, mn, mx);
      }
    }
  }
}

static int launch_group_chunks(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint32_t groups = cql_word(a, 0), per_chunk = cql_word(a, 2);
  if (groups == 0) return 0;
  if (per_chunk == 0 || a.bytes[0] < (uint64_t)groups * 4 || a.bytes[1] < (uint64_t)groups * 4) return (int)cudaErrorInvalidValue;
  k_group_chunks<<<cql_stream_grid((groups + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, groups, per_chunk);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_slot_cursor(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t slots = cql_word(a, 0);
  if (slots == 0) return 0;
  uint32_t groups = (uint32_t)(a.bytes[2] / 4);
  if (a.bytes[0] < slots * 4 || a.bytes[1] < slots * 4 || a.bytes[3] < slots * 4) return (int)cudaErrorInvalidValue;
  k_slot_cursor<<<cql_stream_grid((slots + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, slots, groups);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_chunk_ranges(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint32_t groups = cql_word(a, 0), per_chunk = cql_word(a, 2);
  if (groups == 0) return 0;
  uint64_t cap = std::min(a.bytes[3] / 8, a.bytes[4] / 4);
  if (per_chunk == 0 || a.bytes[0] < (uint64_t)groups * 4 || a.bytes[1] < (uint64_t)groups * 4 || a.bytes[2] < ((uint64_t)groups + 1) * 4)
    return (int)cudaErrorInvalidValue;
  k_chunk_ranges<<<cql_stream_grid(((uint64_t)groups * 32 + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, groups, per_chunk, cap);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_group_fold(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint32_t groups = cql_word(a, 0), exprs = cql_word(a, 2), codes = cql_word(a, 4);
  if (groups == 0) return 0;
  if (exprs == 0 || exprs > 8 || a.bytes[1] < ((uint64_t)groups + 1) * 4 || a.bytes[2] < (uint64_t)groups * exprs * 8) return (int)cudaErrorInvalidValue;
  k_group_fold<<<cql_stream_grid(((uint64_t)groups + HASH_THREADS - 1) / HASH_THREADS, 8), HASH_THREADS, 0, stream>>>(a, groups, exprs, codes);
  CQL_LAUNCH_CHECK();
  return 0;
}

const CqlKernelDesc cql_kernels_hash[] = {
  { "cql_group_chunks", launch_group_chunks },
  { "cql_slot_cursor", launch_slot_cursor },
  { "cql_chunk_ranges", launch_chunk_ranges },
  { "cql_group_fold", launch_group_fold },
  { "aggregate_assign", launch_aggregate_assign },
  { "aggregate_compact", launch_aggregate_compact },
  { "aggregate_hash_reduce_fixed", launch_hash_reduce_fixed },
  { "csr_scatter", launch_csr_scatter },
  { "csr_scatter_tiled", launch_csr_scatter },
  { "aggregate_reduce", launch_aggregate_reduce },
  { "cql_gather_columns", launch_gather_columns },
  { "cql_finite_magnitude", launch_finite_magnitude },
  { "cql_group_small", launch_group_small },
  { "cql_group_direct", launch_group_direct },
  { "cql_group_direct_bits", launch_group_direct_bits },
  { "cql_group_direct_emit", launch_group_direct_emit },
  { "cql_group_finish", launch_group_finish },
  { "cql_gather_string_lengths", launch_gather_string_lengths },
  { "cql_gather_string_bytes", launch_gather_string_bytes },
  { "selection_gather", launch_selection_gather },
  { "cql_widen_f64", launch_widen_f64 },
  { nullptr, nullptr },
};
