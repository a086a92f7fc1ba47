// ORDER BY: an LSD radix sort of (key, position) pairs, the replacement of the reference's bitonic sorts
// (src/gpu/vulkan/shaders/bitonic_sort*.comp, the generated tiled sort query_kernel.c:2114-2267, driven by
// qe_sort_rows, src/query_exec/query_exec.c:5376-6155).
//
// The reference orders rows by up to 4 keys with ties broken by input position. Here every key is turned
// into an unsigned word whose order is the key's order (sign bits flipped, negative floats complemented,
// -0.0 taken as +0.0, complemented again for DESC), and the keys are sorted least significant first with
// a stable radix sort starting from the identity permutation, so equal keys keep their input order.
// Keys of 32-bit columns travel as 4-byte words, the others as 8-byte words.
//
//  cql_sort_keys      binding 0 source column, 1 permutation (u32), 2 key out, 3 selection (u32 rows);
//                     word 0 n, word 2 the CQL type, word 4 descending, word 6 1 = gather through the
//                     permutation, word 8 1 = the n positions are the selection's rows, word 10 the
//                     column's narrow width (0 full, 1 u8 codes, 2 u16 codes, 3 the row number), word 12
//                     the narrow base (value = base + code, in 32 bits)
//  cql_radix_count    binding 0 keys, 1 histogram [256][tiles]; word 0 n, word 2 bit shift, word 4 key bytes
//  cql_radix_scatter  binding 0 keys in, 1 positions in, 2 keys out, 3 positions out, 4 scanned histogram,
//                     5 selection; word 0 n, word 2 bit shift, word 4 key bytes, word 6 1 = write the
//                     selection's row instead of the position, word 8 1 = write no keys (the last pass)
//  cql_pairs_unpack   binding 0 records (u32 words), 1 first out, 2 second out; word 0 n, word 2 words per
//                     record, word 4 the first's word offset, word 6 the second's
//  cql_pairs_pack     binding 0 sorted positions, 1 first, 2 second, 3 pairs out (first, second); word 0 n
//                     (result pairs - join or scan output - put in order on the device by the sort above)
//
// A tile is 8 warps x 16 rounds x 32 rows = 4096 rows. The scatter ranks a row within its tile in input
// order: eight ballots find the lanes of a round with the same digit, per-warp digit counters carry
// the rounds, and a prefix over the warps orders the warps; the global base of (digit, tile) comes from
// an exclusive scan of the digit-major histogram (the prefix_sum kernel).
#include "cql_internal.cuh"
#include <algorithm>

#define SORT_THREADS 256
#define SORT_WARPS (SORT_THREADS / 32)
#define SORT_ROUNDS 16
#define SORT_TILE (SORT_THREADS * SORT_ROUNDS)
#define RADIX 256

__device__ __forceinline__ unsigned long long f64_order(unsigned long long b)
{
  if ((b << 1) == 0) b = 0;  // -0.0 sorts as +0.0
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

// The reference compares every numeric key as an F64 (qe_sort_rows_compare_ctx, query_exec.c:4859-4882):
// 32-bit keys convert exactly, 64-bit integers are rounded to the nearest double first so that values
// that meet in F64 tie (and fall back to their position) as they do there.
__device__ __forceinline__ unsigned long long order_key(uint32_t type, const uint32_t* src, uint64_t i)
{
  const unsigned long long* src64 = (const unsigned long long*)src;
  switch (type)
  {
    case 1: case 12: return src[i];
    case 7: case 9: return src[i] ^ 0x80000000u;
    case 3:
    {
      uint32_t b = src[i];
      if ((b << 1) == 0) b = 0;
      return (b & 0x80000000u) ? (~b & 0xffffffffu) : (b | 0x80000000u);
    }
    case 4: return f64_order(src64[i]);
    case 2: return f64_order(__double_as_longlong((double)src64[i]));
    default: return f64_order(__double_as_longlong((double)(long long)src64[i]));
  }
}

template <typename K>
__global__ void __launch_bounds__(SORT_THREADS) k_sort_keys(CqlLaunch a, uint64_t n, uint64_t src_rows)
{
  const uint32_t* src = (const uint32_t*)a.buf[0];
  uint32_t* perm = (uint32_t*)a.buf[1];
  K* keys = (K*)a.buf[2];
  const uint32_t* sel = (const uint32_t*)a.buf[3];
  uint32_t type = cql_word(a, 2);
  bool desc = cql_word(a, 4) != 0, gather = cql_word(a, 6) != 0, selected = cql_word(a, 8) != 0;
  uint32_t width = cql_word(a, 10), base = cql_word(a, 12);
  uint32_t flip = (type == 7 || type == 9) ? 0x80000000u : 0u;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint64_t p = gather ? perm[i] : i;
    if (!gather) perm[i] = (uint32_t)i;
    uint64_t r = selected ? sel[p] : p;
    unsigned long long k = 0ull;
    if (r < src_rows)
    {
      if (width == 0) k = order_key(type, src, r);
      else
      {
        uint32_t code = width == 1 ? ((const uint8_t*)src)[r] : width == 2 ? ((const uint16_t*)src)[r] : (uint32_t)r;
        k = (base + code) ^ flip;
      }
    }
    if (desc) k = ~k;
    keys[i] = (K)k;
  }
}

template <typename K>
__global__ void __launch_bounds__(SORT_THREADS) k_radix_count(CqlLaunch a, uint64_t n, uint32_t tiles)
{
  // one histogram per warp (fewer lanes on one shared counter), summed at the end of the tile
  __shared__ uint32_t hist[SORT_WARPS][RADIX];
  const K* keys = (const K*)a.buf[0];
  uint32_t* out = (uint32_t*)a.buf[1];
  uint32_t shift = cql_word(a, 2);
  uint32_t warp = threadIdx.x >> 5;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x)
  {
    for (uint32_t i = threadIdx.x; i < SORT_WARPS * RADIX; i += SORT_THREADS) (&hist[0][0])[i] = 0;
    __syncthreads();
    uint64_t base = (uint64_t)tile * SORT_TILE;
    K k[SORT_ROUNDS];
#pragma unroll
    for (uint32_t j = 0; j < SORT_ROUNDS; j++)
    {
      uint64_t i = base + (uint64_t)j * SORT_THREADS + threadIdx.x;
      k[j] = i < n ? keys[i] : (K)0;
    }
#pragma unroll
    for (uint32_t j = 0; j < SORT_ROUNDS; j++)
    {
      uint64_t i = base + (uint64_t)j * SORT_THREADS + threadIdx.x;
      if (i < n) atomicAdd(&hist[warp][(uint32_t)(k[j] >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    for (uint32_t d = threadIdx.x; d < RADIX; d += SORT_THREADS)
    {
      uint32_t total = 0;
#pragma unroll
      for (uint32_t w = 0; w < SORT_WARPS; w++) total += hist[w][d];
      out[(uint64_t)d * tiles + tile] = total;
    }
    __syncthreads();
  }
}

// The scatter of one tile: rank every key within the tile in input order (per-warp counters, lanes of
// one digit found by ballots), place the tile in shared memory in digit order, then write
// it out in that order, so consecutive threads write consecutive places of each digit's run.
//
// The kernel is bound by the latency of the ranking's shared-memory chain, so it is built for several
// resident CTAs per SM: only the keys and their ranks live in registers while a tile is ranked (the
// positions are read once the ranks are known), within the register budget of 4 CTAs (3 for 8-byte keys).
#define SORT_SCATTER_CTAS(K) (sizeof(K) == 4 ? 4 : 3)

// The lanes of the warp whose digit equals this lane's, from one ballot per digit bit (the match
// instruction is far slower); a ninth bit marks the lanes past the end in the last, partial tile.
__device__ __forceinline__ uint32_t same_digit_lanes(uint32_t dg, bool partial)
{
  uint32_t peers = 0xffffffffu;
#pragma unroll
  for (uint32_t b = 0; b < 8; b++)
  {
    uint32_t bit = (dg >> b) & 1u;
    uint32_t m = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? m : ~m;
  }
  if (partial)
  {
    uint32_t bit = (dg >> 8) & 1u;
    uint32_t m = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? m : ~m;
  }
  return peers;
}

template <typename K>
__global__ void __launch_bounds__(SORT_THREADS, SORT_SCATTER_CTAS(K)) k_radix_scatter(CqlLaunch a, uint64_t n, uint32_t tiles)
{
  __shared__ uint32_t warp_count[SORT_WARPS][RADIX];
  __shared__ uint32_t s_start[RADIX];    // place of each digit's first key inside the tile
  __shared__ uint32_t s_off[RADIX];      // global place of a tile place j of the digit: s_off + j (mod 2^32)
  __shared__ uint32_t s_warp_total[SORT_WARPS];
  extern __shared__ __align__(16) unsigned char s_tile[];
  K* s_key = (K*)s_tile;
  uint32_t* s_pos = (uint32_t*)(s_tile + sizeof(K) * SORT_TILE);
  const K* keys_in = (const K*)a.buf[0];
  const uint32_t* pos_in = (const uint32_t*)a.buf[1];
  K* keys_out = (K*)a.buf[2];
  uint32_t* pos_out = (uint32_t*)a.buf[3];
  const uint32_t* base_of = (const uint32_t*)a.buf[4];
  const uint32_t* sel = (const uint32_t*)a.buf[5];
  uint32_t shift = cql_word(a, 2);
  bool map_rows = cql_word(a, 6) != 0, write_keys = cql_word(a, 8) == 0;
  uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t lt = (1u << lane) - 1u;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x)
  {
    for (uint32_t i = threadIdx.x; i < SORT_WARPS * RADIX; i += SORT_THREADS) (&warp_count[0][0])[i] = 0;
    // each warp owns 16 rounds of 32 consecutive rows; its keys are loaded up front
    uint64_t tile_first = (uint64_t)tile * SORT_TILE;
    uint32_t tile_rows = (uint32_t)min((uint64_t)SORT_TILE, n - tile_first);
    bool partial = tile_rows != SORT_TILE;
    uint64_t warp_base = tile_first + (uint64_t)warp * 32 * SORT_ROUNDS;
    K key[SORT_ROUNDS];
#pragma unroll
    for (uint32_t r = 0; r < SORT_ROUNDS; r++)
    {
      uint64_t i = warp_base + (uint64_t)r * 32 + lane;
      key[r] = i < n ? keys_in[i] : (K)0;
    }
    uint32_t d = threadIdx.x;
    uint32_t tile_base = base_of[(uint64_t)d * tiles + tile];
    __syncthreads();
    uint32_t local[SORT_ROUNDS];
#pragma unroll
    for (uint32_t r = 0; r < SORT_ROUNDS; r++)
    {
      uint64_t i = warp_base + (uint64_t)r * 32 + lane;
      uint32_t dg = i < n ? ((uint32_t)(key[r] >> shift) & 0xffu) : RADIX;  // RADIX: past the end
      uint32_t peers = same_digit_lanes(dg, partial);
      uint32_t before = dg < RADIX ? warp_count[warp][dg] : 0u;
      local[r] = before + __popc(peers & lt);
      __syncwarp();
      if (dg < RADIX && (peers & lt) == 0) warp_count[warp][dg] = before + __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    // per digit (one per thread): the warps before each warp, and the digit's total in the tile
    uint32_t run = 0;
#pragma unroll
    for (uint32_t w = 0; w < SORT_WARPS; w++)
    {
      uint32_t c = warp_count[w][d];
      warp_count[w][d] = run;
      run += c;
    }
    // exclusive scan of the digit totals over the block: where each digit starts in the tile
    uint32_t incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) s_warp_total[warp] = incl;
    __syncthreads();
    uint32_t warp_prefix = 0;
    for (uint32_t w = 0; w < warp; w++) warp_prefix += s_warp_total[w];
    uint32_t start = warp_prefix + incl - run;
    s_start[d] = start;
    s_off[d] = tile_base - start;
    __syncthreads();
    // the tile in digit order, in shared memory: the keys, then the positions read now
#pragma unroll
    for (uint32_t r = 0; r < SORT_ROUNDS; r++)
    {
      uint64_t i = warp_base + (uint64_t)r * 32 + lane;
      uint32_t dg = (uint32_t)(key[r] >> shift) & 0xffu;
      local[r] += s_start[dg] + warp_count[warp][dg];
      if (i < n) s_key[local[r]] = key[r];
    }
    uint32_t pos[SORT_ROUNDS];
#pragma unroll
    for (uint32_t r = 0; r < SORT_ROUNDS; r++)
    {
      uint64_t i = warp_base + (uint64_t)r * 32 + lane;
      pos[r] = i < n ? pos_in[i] : 0u;
    }
#pragma unroll
    for (uint32_t r = 0; r < SORT_ROUNDS; r++)
    {
      uint64_t i = warp_base + (uint64_t)r * 32 + lane;
      if (i < n) s_pos[local[r]] = pos[r];
    }
    __syncthreads();
    // out in order: place j of the tile goes to its digit's global base plus its place in the run
    for (uint32_t j = threadIdx.x; j < tile_rows; j += SORT_THREADS)
    {
      K k = s_key[j];
      uint32_t dd = (uint32_t)(k >> shift) & 0xffu;
      uint64_t dst = (uint32_t)(s_off[dd] + j);
      if (dst < n)
      {
        if (write_keys) keys_out[dst] = k;
        uint32_t p = s_pos[j];
        pos_out[dst] = map_rows ? sel[p] : p;
      }
    }
    __syncthreads();
  }
}

static bool sort_type_wide_host(uint32_t type)
{
  return type == 2 || type == 4 || type == 8 || type == 10 || type == 11;
}

static int sort_key_bytes(uint32_t type)
{
  switch (type)
  {
    case 1: case 3: case 7: case 9: case 12: return 4;
    case 2: case 4: case 8: case 10: case 11: return 8;
    default: return 0;
  }
}

static int launch_sort_keys(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t n = cql_word(a, 0);
  uint32_t type = cql_word(a, 2);
  int kb = sort_key_bytes(type);
  if (n == 0) return 0;
  if (!kb || a.bytes[1] < n * 4 || a.bytes[2] < n * (uint64_t)kb) return (int)cudaErrorInvalidValue;
  if (cql_word(a, 8) && a.bytes[3] < n * 4) return (int)cudaErrorInvalidValue;
  uint32_t width = cql_word(a, 10);
  if (width > 3 || (width && sort_type_wide_host(type))) return (int)cudaErrorInvalidValue;
  uint64_t src_rows = width == 3 ? ~0ull : width ? a.bytes[0] / width : a.bytes[0] / (sort_type_wide_host(type) ? 8 : 4);
  uint32_t grid = cql_stream_grid((n + SORT_THREADS - 1) / SORT_THREADS, 8);
  if (kb == 4) k_sort_keys<uint32_t><<<grid, SORT_THREADS, 0, stream>>>(a, n, src_rows);
  else k_sort_keys<unsigned long long><<<grid, SORT_THREADS, 0, stream>>>(a, n, src_rows);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_radix_count(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t n = cql_word(a, 0);
  uint32_t shift = cql_word(a, 2), kb = cql_word(a, 4);
  if (n == 0) return 0;
  uint32_t tiles = (uint32_t)((n + SORT_TILE - 1) / SORT_TILE);
  if ((kb != 4 && kb != 8) || shift >= kb * 8 || a.bytes[0] < n * kb || (uint64_t)tiles * RADIX * 4 > a.bytes[1])
    return (int)cudaErrorInvalidValue;
  uint32_t grid = cql_stream_grid(tiles, 8);
  if (kb == 4) k_radix_count<uint32_t><<<grid, SORT_THREADS, 0, stream>>>(a, n, tiles);
  else k_radix_count<unsigned long long><<<grid, SORT_THREADS, 0, stream>>>(a, n, tiles);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_radix_scatter(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t n = cql_word(a, 0);
  uint32_t shift = cql_word(a, 2), kb = cql_word(a, 4);
  if (n == 0) return 0;
  uint32_t tiles = (uint32_t)((n + SORT_TILE - 1) / SORT_TILE);
  bool write_keys = cql_word(a, 8) == 0;
  if ((kb != 4 && kb != 8) || shift >= kb * 8 || a.bytes[0] < n * kb || a.bytes[1] < n * 4 || a.bytes[3] < n * 4 ||
      (write_keys && a.bytes[2] < n * kb) || (uint64_t)tiles * RADIX * 4 > a.bytes[4] || (cql_word(a, 6) && a.bytes[5] < n * 4))
    return (int)cudaErrorInvalidValue;
  // the tile's keys and positions staged in dynamic shared memory
  size_t smem = (size_t)SORT_TILE * (kb + 4);
  const void* fn = kb == 4 ? (const void*)k_radix_scatter<uint32_t> : (const void*)k_radix_scatter<unsigned long long>;
  // dynamic plus static shared memory passes the default 48 KB for 8-byte keys: opt in
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  int per_sm = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, SORT_THREADS, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
  uint32_t grid = cql_stream_grid(tiles, per_sm);
  if (kb == 4) k_radix_scatter<uint32_t><<<grid, SORT_THREADS, smem, stream>>>(a, n, tiles);
  else k_radix_scatter<unsigned long long><<<grid, SORT_THREADS, smem, stream>>>(a, n, tiles);
  CQL_LAUNCH_CHECK();
  return 0;
}

__global__ void k_pairs_unpack(CqlLaunch a, uint64_t n, uint32_t stride, uint32_t fa, uint32_t fb)
{
  const uint32_t* rec = (const uint32_t*)a.buf[0];
  uint32_t* first = (uint32_t*)a.buf[1];
  uint32_t* second = (uint32_t*)a.buf[2];
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    first[i] = rec[i * stride + fa];
    second[i] = rec[i * stride + fb];
  }
}

__global__ void k_pairs_pack(CqlLaunch a, uint64_t n)
{
  const uint32_t* order = (const uint32_t*)a.buf[0];
  const uint32_t* first = (const uint32_t*)a.buf[1];
  const uint32_t* second = (const uint32_t*)a.buf[2];
  uint2* out = (uint2*)a.buf[3];
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t p = order[i];
    out[i] = make_uint2(first[p], second[p]);
  }
}

static int launch_pairs_unpack(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t n = cql_word(a, 0);
  uint32_t stride = cql_word(a, 2), fa = cql_word(a, 4), fb = cql_word(a, 6);
  if (n == 0) return 0;
  if (stride == 0 || fa >= stride || fb >= stride || a.bytes[0] < n * stride * 4 || a.bytes[1] < n * 4 || a.bytes[2] < n * 4)
    return (int)cudaErrorInvalidValue;
  k_pairs_unpack<<<cql_stream_grid((n + SORT_THREADS - 1) / SORT_THREADS, 8), SORT_THREADS, 0, stream>>>(a, n, stride, fa, fb);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_pairs_pack(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t n = cql_word(a, 0);
  if (n == 0) return 0;
  if (a.bytes[0] < n * 4 || a.bytes[1] < n * 4 || a.bytes[2] < n * 4 || a.bytes[3] < n * 8) return (int)cudaErrorInvalidValue;
  k_pairs_pack<<<cql_stream_grid((n + SORT_THREADS - 1) / SORT_THREADS, 8), SORT_THREADS, 0, stream>>>(a, n);
  CQL_LAUNCH_CHECK();
  return 0;
}

const CqlKernelDesc cql_kernels_sort[] = {
  { "cql_pairs_unpack", launch_pairs_unpack },
  { "cql_pairs_pack", launch_pairs_pack },
  { "cql_sort_keys", launch_sort_keys },
  { "cql_radix_count", launch_radix_count },
  { "cql_radix_scatter", launch_radix_scatter },
  { nullptr, nullptr },
};
