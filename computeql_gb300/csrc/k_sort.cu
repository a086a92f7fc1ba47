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
//  cql_sort_keys      binding 0 source column, 1 permutation (u32), 2 key out, 3 selection (u32 rows),
//                     4 histogram [256][tiles] of the first digit, 5 digit totals [key bytes][256] (4 and 5
//                     with word 14 = 1); word 0 n, word 2 the CQL type, word 4 descending, word 6 1 = gather
//                     through the permutation, word 8 1 = the n positions are the selection's rows, word 10
//                     the column's narrow width (0 full, 1 u8 codes, 2 u16 codes, 3 the row number), word 12
//                     the narrow base (value = base + code, in 32 bits), word 14 flags: 1 = count the first
//                     digit, 2 = write no identity permutation (the first scatter takes row numbers)
//  cql_radix_count    binding 0 keys, 1 histogram [256][tiles], 2 the pass's digit totals [256] (added to);
//                     word 0 n, word 2 bit shift, word 4 key bytes
//  cql_radix_offsets  binding 0 histogram [256][tiles], 1 the pass's digit totals [256], 2 offsets out
//                     [256][tiles] (where each (digit, tile) run starts in the pass's output); word 0 n
//  cql_radix_scatter  binding 0 keys in, 1 positions in, 2 keys out, 3 positions out, 4 offsets,
//                     5 selection; word 0 n, word 2 bit shift, word 4 key bytes, word 6 1 = write the
//                     selection's row instead of the position, word 8 1 = write no keys (the last pass),
//                     word 10 1 = the positions in are the row numbers (binding 1 is not read); binding 6
//                     (optional) the pass's digit totals: one digit holding all n rows makes the pass a copy
//  cql_pairs_unpack   binding 0 records (u32 words), 1 first out, 2 second out; word 0 n, word 2 words per
//                     record, word 4 the first's word offset, word 6 the second's
//  cql_pairs_pack     binding 0 sorted positions, 1 first, 2 second, 3 pairs out (first, second); word 0 n
//                     (result pairs - join or scan output - put in order on the device by the sort above)
//
// A tile is 8 warps x 16 rounds x 32 rows = 4096 rows. The scatter ranks a row within its tile in input
// order: eight ballots or the match instruction (alternate rounds) find the lanes of a round with the same
// digit, per-warp digit counters carry the rounds, and a prefix over the warps orders the warps; the global
// base of (digit, tile) comes from the offsets kernel: the digit's place in the pass's output (the totals of the digits below it, counted
// while the histogram is made) plus the digit's counts in the tiles before.
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
__device__ __forceinline__ unsigned long long order_bits(uint32_t type, unsigned long long raw)
{
  switch (type)
  {
    case 1: case 12: return (uint32_t)raw;
    case 7: case 9: return (uint32_t)raw ^ 0x80000000u;
    case 3:
    {
      uint32_t b = (uint32_t)raw;
      if ((b << 1) == 0) b = 0;
      return (b & 0x80000000u) ? (~b & 0xffffffffu) : (b | 0x80000000u);
    }
    case 4: return f64_order(raw);
    case 2: return f64_order(__double_as_longlong((double)raw));
    default: return f64_order(__double_as_longlong((double)(long long)raw));
  }
}

// Counts digits into a histogram a run of equal digits at a time: one shared atomic per run, so a digit
// that does not vary (the high bytes of small keys, the low bytes of whole-number doubles) costs one atomic
// per thread and tile instead of 32 lanes meeting on one counter for every row.
struct DigitRun
{
  uint32_t digit = 0xffffffffu, count = 0;
  __device__ __forceinline__ void add(uint32_t* hist, uint32_t dg)
  {
    if (dg != digit)
    {
      if (count) atomicAdd(&hist[digit], count);
      digit = dg;
      count = 0;
    }
    count += 1;
  }
  __device__ __forceinline__ void flush(uint32_t* hist)
  {
    if (count) atomicAdd(&hist[digit], count);
  }
};

// The keys of one tile in sort order; with COUNT, the first digit counted into the warp's histogram. The
// source rows are found first, then the values read (16 loads in flight a thread), then turned into keys.
template <typename K, bool PARTIAL, bool COUNT>
__device__ __forceinline__ void keys_tile(const CqlLaunch& a, uint64_t n, uint64_t src_rows, uint32_t tile, uint32_t* warp_hist)
{
  const uint32_t* src = (const uint32_t*)a.buf[0];
  uint32_t* perm = (uint32_t*)a.buf[1];
  K* keys = (K*)a.buf[2];
  const uint32_t* sel = (const uint32_t*)a.buf[3];
  uint32_t type = cql_word(a, 2);
  bool desc = cql_word(a, 4) != 0, gather = cql_word(a, 6) != 0, selected = cql_word(a, 8) != 0;
  bool write_identity = !gather && (cql_word(a, 14) & 2u) == 0;
  uint32_t width = cql_word(a, 10), base = cql_word(a, 12);
  uint32_t flip = (type == 7 || type == 9) ? 0x80000000u : 0u;
  uint64_t first = (uint64_t)tile * SORT_TILE;
  uint32_t rows = PARTIAL ? (uint32_t)(n - first) : SORT_TILE;
  uint32_t row[SORT_ROUNDS];
#pragma unroll
  for (uint32_t j = 0; j < SORT_ROUNDS; j++)
  {
    uint32_t o = j * SORT_THREADS + threadIdx.x;
    uint32_t p = (uint32_t)(first + o);
    if (gather && (!PARTIAL || o < rows)) p = perm[first + o];
    row[j] = p;
  }
  if (selected)
  {
#pragma unroll
    for (uint32_t j = 0; j < SORT_ROUNDS; j++)
      if (!PARTIAL || j * SORT_THREADS + threadIdx.x < rows) row[j] = sel[row[j]];
  }
  if (write_identity)
  {
#pragma unroll
    for (uint32_t j = 0; j < SORT_ROUNDS; j++)
    {
      uint32_t o = j * SORT_THREADS + threadIdx.x;
      if (!PARTIAL || o < rows) perm[first + o] = (uint32_t)(first + o);
    }
  }
  K raw[SORT_ROUNDS];
#pragma unroll
  for (uint32_t j = 0; j < SORT_ROUNDS; j++)
  {
    uint32_t o = j * SORT_THREADS + threadIdx.x;
    uint32_t r = row[j];
    K v = 0;
    if ((!PARTIAL || o < rows) && r < src_rows)
    {
      if (sizeof(K) == 8) v = (K)((const unsigned long long*)src)[r];
      else if (width == 0) v = (K)src[r];
      else if (width == 1) v = (K)((const uint8_t*)src)[r];
      else if (width == 2) v = (K)((const uint16_t*)src)[r];
      else v = (K)r;
    }
    raw[j] = v;
  }
  DigitRun run;
#pragma unroll
  for (uint32_t j = 0; j < SORT_ROUNDS; j++)
  {
    uint32_t o = j * SORT_THREADS + threadIdx.x;
    if (PARTIAL && o >= rows) continue;
    unsigned long long k = 0ull;
    if (row[j] < src_rows) k = width == 0 ? order_bits(type, raw[j]) : (unsigned long long)(((uint32_t)raw[j] + base) ^ flip);
    if (desc) k = ~k;
    keys[first + o] = (K)k;
    if (COUNT) run.add(warp_hist, (uint32_t)k & 0xffu);
  }
  if (COUNT) run.flush(warp_hist);
}

template <typename K, bool COUNT>
__global__ void __launch_bounds__(SORT_THREADS) k_sort_keys(CqlLaunch a, uint64_t n, uint64_t src_rows, uint32_t tiles)
{
  __shared__ uint32_t hist[COUNT ? SORT_WARPS : 1][RADIX];
  uint32_t* hist_out = (uint32_t*)a.buf[4];
  uint32_t* totals = (uint32_t*)a.buf[5];
  uint32_t warp = threadIdx.x >> 5, d = threadIdx.x;  // RADIX == SORT_THREADS: thread d sums digit d
  uint32_t full_tiles = (uint32_t)(n / SORT_TILE), cta_total = 0;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x)
  {
    if (COUNT)
    {
      for (uint32_t i = threadIdx.x; i < SORT_WARPS * RADIX; i += SORT_THREADS) (&hist[0][0])[i] = 0;
      __syncthreads();
    }
    if (tile < full_tiles) keys_tile<K, false, COUNT>(a, n, src_rows, tile, hist[COUNT ? warp : 0]);
    else keys_tile<K, true, COUNT>(a, n, src_rows, tile, hist[COUNT ? warp : 0]);
    if (COUNT)
    {
      __syncthreads();
      uint32_t total = 0;
#pragma unroll
      for (uint32_t w = 0; w < SORT_WARPS; w++) total += hist[w][d];
      hist_out[(uint64_t)d * tiles + tile] = total;
      cta_total += total;
      __syncthreads();
    }
  }
  if (COUNT && cta_total) atomicAdd(&totals[d], cta_total);
}

template <typename K, bool PARTIAL>
__device__ __forceinline__ void count_tile(const K* keys, uint64_t n, uint32_t tile, uint32_t shift, uint32_t* warp_hist)
{
  uint64_t first = (uint64_t)tile * SORT_TILE;
  const K* kin = keys + first;
  uint32_t rows = PARTIAL ? (uint32_t)(n - first) : SORT_TILE;
  K k[SORT_ROUNDS];
#pragma unroll
  for (uint32_t j = 0; j < SORT_ROUNDS; j++)
  {
    uint32_t o = j * SORT_THREADS + threadIdx.x;
    k[j] = (!PARTIAL || o < rows) ? kin[o] : (K)0;
  }
  DigitRun run;
#pragma unroll
  for (uint32_t j = 0; j < SORT_ROUNDS; j++)
    if (!PARTIAL || j * SORT_THREADS + threadIdx.x < rows) run.add(warp_hist, (uint32_t)(k[j] >> shift) & 0xffu);
  run.flush(warp_hist);
}

template <typename K>
__global__ void __launch_bounds__(SORT_THREADS) k_radix_count(CqlLaunch a, uint64_t n, uint32_t tiles)
{
  // one histogram per warp (fewer lanes on one shared counter), summed at the end of the tile
  __shared__ uint32_t hist[SORT_WARPS][RADIX];
  const K* keys = (const K*)a.buf[0];
  uint32_t* out = (uint32_t*)a.buf[1];
  uint32_t* totals = (uint32_t*)a.buf[2];
  uint32_t shift = cql_word(a, 2);
  uint32_t warp = threadIdx.x >> 5, d = threadIdx.x;
  uint32_t full_tiles = (uint32_t)(n / SORT_TILE);
  uint32_t cta_total = 0;  // digit d's count over this CTA's tiles (RADIX == SORT_THREADS)
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x)
  {
    for (uint32_t i = threadIdx.x; i < SORT_WARPS * RADIX; i += SORT_THREADS) (&hist[0][0])[i] = 0;
    __syncthreads();
    if (tile < full_tiles) count_tile<K, false>(keys, n, tile, shift, hist[warp]);
    else count_tile<K, true>(keys, n, tile, shift, hist[warp]);
    __syncthreads();
    uint32_t total = 0;
#pragma unroll
    for (uint32_t w = 0; w < SORT_WARPS; w++) total += hist[w][d];
    out[(uint64_t)d * tiles + tile] = total;
    cta_total += total;
    __syncthreads();
  }
  if (cta_total) atomicAdd(&totals[d], cta_total);
}

// Where each (digit, tile) run starts in the pass's output: one CTA a digit, the totals of the digits below
// it plus an exclusive scan of its row of the histogram (4 counts a thread, 2048 a step).
#define OFFSETS_THREADS 512
__global__ void __launch_bounds__(OFFSETS_THREADS) k_radix_offsets(CqlLaunch a, uint32_t tiles)
{
  __shared__ uint32_t s_warp[OFFSETS_THREADS / 32];
  const uint32_t* hist = (const uint32_t*)a.buf[0];
  const uint32_t* totals = (const uint32_t*)a.buf[1];
  uint32_t* out = (uint32_t*)a.buf[2];
  uint32_t d = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t below = threadIdx.x < d ? totals[threadIdx.x] : 0u;  // d < RADIX <= OFFSETS_THREADS
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) below += __shfl_xor_sync(0xffffffffu, below, o);
  if (lane == 0) s_warp[warp] = below;
  __syncthreads();
  uint32_t carry = 0;
#pragma unroll
  for (uint32_t w = 0; w < OFFSETS_THREADS / 32; w++) carry += s_warp[w];
  __syncthreads();
  const uint32_t* row = hist + (uint64_t)d * tiles;
  uint32_t* orow = out + (uint64_t)d * tiles;
  for (uint32_t start = 0; start < tiles; start += OFFSETS_THREADS * 4)
  {
    uint32_t j0 = start + threadIdx.x * 4;
    uint32_t v[4], t = 0;
#pragma unroll
    for (uint32_t q = 0; q < 4; q++)
    {
      v[q] = j0 + q < tiles ? row[j0 + q] : 0u;
      t += v[q];
    }
    uint32_t incl = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    uint32_t before = 0, step = 0;
#pragma unroll
    for (uint32_t w = 0; w < OFFSETS_THREADS / 32; w++)
    {
      uint32_t c = s_warp[w];
      before += w < warp ? c : 0u;
      step += c;
    }
    uint32_t at = carry + before + incl - t;
#pragma unroll
    for (uint32_t q = 0; q < 4; q++)
    {
      if (j0 + q < tiles) orow[j0 + q] = at;
      at += v[q];
    }
    carry += step;
    __syncthreads();
  }
}

// The scatter of one tile: rank every key within the tile in input order (per-warp counters, lanes of
// one digit found within each 32-row round), place the tile in shared memory in digit order, then write
// it out in that order, so consecutive threads write consecutive places of each digit's run.
//
// The ranking is bound by instruction issue and the latency of its shared-memory chain, so the kernel is
// built for several resident CTAs per SM: only the keys and their ranks live in registers while a tile is
// ranked (the positions are read once the ranks are known), within the register budget of 4 CTAs (3 for
// 8-byte keys). Full tiles take a path without bounds checks; the last, partial tile the checked one.
#define SORT_SCATTER_CTAS(K) (sizeof(K) == 4 ? 4 : 3)

// Ranking forms: the lanes of a round with the same digit found by eight ballots (ALU pipe), by the match
// instruction (its own, slower pipe), or the two in alternate rounds so that both pipes share the work.
#define RANK_BALLOTS 0
#define RANK_MATCH 1
#define RANK_ALTERNATE 2
#ifndef SORT_RANK_FORM
#define SORT_RANK_FORM RANK_ALTERNATE
#endif

// The lanes of the warp whose digit equals this lane's, from one ballot per digit bit; a ninth bit marks
// the lanes past the end in the last, partial tile.
template <bool PARTIAL>
__device__ __forceinline__ uint32_t same_digit_lanes(uint32_t dg)
{
  uint32_t peers = 0xffffffffu;
#pragma unroll
  for (uint32_t b = 0; b < (PARTIAL ? 9u : 8u); b++)
  {
    uint32_t bit = (dg >> b) & 1u;
    uint32_t m = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? m : ~m;
  }
  return peers;
}

template <int FORM, bool PARTIAL>
__device__ __forceinline__ uint32_t round_peers(uint32_t dg, uint32_t r)
{
  if (FORM == RANK_MATCH || (FORM == RANK_ALTERNATE && (r & 1u))) return __match_any_sync(0xffffffffu, dg);
  return same_digit_lanes<PARTIAL>(dg);
}

struct ScatterShared
{
  uint32_t warp_count[SORT_WARPS][RADIX];  // per warp and digit: ranked count, then the place of its first key
  uint32_t off[RADIX];                      // global place of tile place j of the digit: off + j (mod 2^32)
  uint32_t warp_total[SORT_WARPS];
};

template <typename K, bool PARTIAL, int FORM>
__device__ __forceinline__ void scatter_tile(const CqlLaunch& a, ScatterShared& sh, K* s_key, uint32_t* s_pos, uint64_t n, uint32_t tiles,
                                             uint32_t tile, uint32_t shift, bool map_rows, bool write_keys, bool identity)
{
  const K* keys_in = (const K*)a.buf[0];
  const uint32_t* pos_in = (const uint32_t*)a.buf[1];
  K* keys_out = (K*)a.buf[2];
  uint32_t* pos_out = (uint32_t*)a.buf[3];
  const uint32_t* base_of = (const uint32_t*)a.buf[4];
  const uint32_t* sel = (const uint32_t*)a.buf[5];
  uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, d = threadIdx.x;
  uint32_t lt = (1u << lane) - 1u;
  for (uint32_t i = threadIdx.x; i < SORT_WARPS * RADIX; i += SORT_THREADS) (&sh.warp_count[0][0])[i] = 0;
  // each warp owns 16 rounds of 32 consecutive rows; its keys are loaded up front
  uint64_t tile_first = (uint64_t)tile * SORT_TILE;
  uint32_t tile_rows = PARTIAL ? (uint32_t)min((uint64_t)SORT_TILE, n - tile_first) : SORT_TILE;
  uint32_t warp_first = warp * 32 * SORT_ROUNDS;  // within the tile
  const K* kin = keys_in + tile_first + warp_first;
  K key[SORT_ROUNDS];
#pragma unroll
  for (uint32_t r = 0; r < SORT_ROUNDS; r++)
  {
    uint32_t j = warp_first + r * 32 + lane;
    key[r] = (!PARTIAL || j < tile_rows) ? kin[r * 32 + lane] : (K)0;
  }
  uint32_t tile_base = base_of[(uint64_t)d * tiles + tile];
  __syncthreads();
  uint32_t local[SORT_ROUNDS];
#pragma unroll
  for (uint32_t r = 0; r < SORT_ROUNDS; r++)
  {
    uint32_t j = warp_first + r * 32 + lane;
    uint32_t dg = (uint32_t)(key[r] >> shift) & 0xffu;
    if (PARTIAL && j >= tile_rows) dg = RADIX;  // past the end
    uint32_t peers = round_peers<FORM, PARTIAL>(dg, r);
    uint32_t before = (!PARTIAL || dg < RADIX) ? sh.warp_count[warp][dg] : 0u;
    local[r] = before + __popc(peers & lt);
    __syncwarp();
    if ((!PARTIAL || dg < RADIX) && (peers & lt) == 0) sh.warp_count[warp][dg] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit (one per thread): the warps before each warp, and the digit's total in the tile
  uint32_t run = 0;
#pragma unroll
  for (uint32_t w = 0; w < SORT_WARPS; w++)
  {
    uint32_t c = sh.warp_count[w][d];
    sh.warp_count[w][d] = run;
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
  if (lane == 31) sh.warp_total[warp] = incl;
  __syncthreads();
  uint32_t start = incl - run;
  for (uint32_t w = 0; w < warp; w++) start += sh.warp_total[w];
  sh.off[d] = tile_base - start;
  // the place in the tile of each warp's first key of the digit
#pragma unroll
  for (uint32_t w = 0; w < SORT_WARPS; w++) sh.warp_count[w][d] += start;
  __syncthreads();
  // the tile in digit order, in shared memory: the keys, then the positions read now
#pragma unroll
  for (uint32_t r = 0; r < SORT_ROUNDS; r++)
  {
    uint32_t j = warp_first + r * 32 + lane;
    uint32_t dg = (uint32_t)(key[r] >> shift) & 0xffu;
    local[r] += sh.warp_count[warp][dg];
    if (!PARTIAL || j < tile_rows) s_key[local[r]] = key[r];
  }
  const uint32_t* pin = pos_in + tile_first + warp_first;
  uint32_t pos[SORT_ROUNDS];
#pragma unroll
  for (uint32_t r = 0; r < SORT_ROUNDS; r++)
  {
    uint32_t j = warp_first + r * 32 + lane;
    pos[r] = identity ? (uint32_t)(tile_first + j) : (!PARTIAL || j < tile_rows) ? pin[r * 32 + lane] : 0u;
  }
#pragma unroll
  for (uint32_t r = 0; r < SORT_ROUNDS; r++)
  {
    uint32_t j = warp_first + r * 32 + lane;
    if (!PARTIAL || j < tile_rows) s_pos[local[r]] = pos[r];
  }
  __syncthreads();
  // out in order: place j of the tile goes to its digit's global base plus its place in the run
#pragma unroll 4
  for (uint32_t j = threadIdx.x; j < tile_rows; j += SORT_THREADS)
  {
    K k = s_key[j];
    uint32_t dd = (uint32_t)(k >> shift) & 0xffu;
    uint64_t dst = (uint32_t)(sh.off[dd] + j);
    if (dst < n)
    {
      if (write_keys) keys_out[dst] = k;
      uint32_t p = s_pos[j];
      pos_out[dst] = map_rows ? sel[p] : p;
    }
  }
  __syncthreads();
}

// A pass whose digit is the same for every row (a byte that does not vary) leaves the order as it is: the
// keys and positions are copied through, with no ranking.
template <typename K>
__device__ __forceinline__ void pass_copy(const CqlLaunch& a, uint64_t n, bool map_rows, bool write_keys, bool identity)
{
  const K* keys_in = (const K*)a.buf[0];
  const uint32_t* pos_in = (const uint32_t*)a.buf[1];
  K* keys_out = (K*)a.buf[2];
  uint32_t* pos_out = (uint32_t*)a.buf[3];
  const uint32_t* sel = (const uint32_t*)a.buf[5];
  uint64_t stride = (uint64_t)gridDim.x * SORT_THREADS;
#pragma unroll 4
  for (uint64_t i = (uint64_t)blockIdx.x * SORT_THREADS + threadIdx.x; i < n; i += stride)
  {
    if (write_keys) keys_out[i] = keys_in[i];
    uint32_t p = identity ? (uint32_t)i : pos_in[i];
    pos_out[i] = map_rows ? sel[p] : p;
  }
}

template <typename K, int FORM>
__global__ void __launch_bounds__(SORT_THREADS, SORT_SCATTER_CTAS(K)) k_radix_scatter(CqlLaunch a, uint64_t n, uint32_t tiles, bool has_totals)
{
  __shared__ ScatterShared sh;
  __shared__ uint32_t s_one_digit;
  extern __shared__ __align__(16) unsigned char s_tile[];
  K* s_key = (K*)s_tile;
  uint32_t* s_pos = (uint32_t*)(s_tile + sizeof(K) * SORT_TILE);
  uint32_t shift = cql_word(a, 2);
  bool map_rows = cql_word(a, 6) != 0, write_keys = cql_word(a, 8) == 0, identity = cql_word(a, 10) != 0;
  if (has_totals)
  {
    // the pass's digit totals: one digit holding every row makes the pass a copy
    const uint32_t* totals = (const uint32_t*)a.buf[6];
    if (threadIdx.x == 0) s_one_digit = 0;
    __syncthreads();
    if (totals[threadIdx.x] == (uint32_t)n) s_one_digit = 1;  // RADIX == SORT_THREADS; n < 2^32
    __syncthreads();
    if (s_one_digit)
    {
      pass_copy<K>(a, n, map_rows, write_keys, identity);
      return;
    }
  }
  uint32_t full_tiles = (uint32_t)(n / SORT_TILE);
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x)
  {
    if (tile < full_tiles) scatter_tile<K, false, FORM>(a, sh, s_key, s_pos, n, tiles, tile, shift, map_rows, write_keys, identity);
    else scatter_tile<K, true, FORM>(a, sh, s_key, s_pos, n, tiles, tile, shift, map_rows, write_keys, identity);
  }
}

// CTAs of SORT_THREADS threads that fit on an SM (1 when the query fails): a tile loop's grid
static int resident_ctas(const void* fn, size_t smem)
{
  int per_sm = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, SORT_THREADS, smem) != cudaSuccess || per_sm < 1)
  {
    cudaGetLastError();
    per_sm = 1;
  }
  return per_sm;
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
  uint32_t tiles = (uint32_t)((n + SORT_TILE - 1) / SORT_TILE);
  bool count = (cql_word(a, 14) & 1u) != 0;
  if (count && ((uint64_t)tiles * RADIX * 4 > a.bytes[4] || a.bytes[5] < RADIX * 4)) return (int)cudaErrorInvalidValue;
  const void* fn = kb == 4 ? (count ? (const void*)k_sort_keys<uint32_t, true> : (const void*)k_sort_keys<uint32_t, false>)
                            : (count ? (const void*)k_sort_keys<unsigned long long, true> : (const void*)k_sort_keys<unsigned long long, false>);
  uint32_t grid = cql_stream_grid(tiles, resident_ctas(fn, 0));
  if (kb == 4)
  {
    if (count) k_sort_keys<uint32_t, true><<<grid, SORT_THREADS, 0, stream>>>(a, n, src_rows, tiles);
    else k_sort_keys<uint32_t, false><<<grid, SORT_THREADS, 0, stream>>>(a, n, src_rows, tiles);
  }
  else
  {
    if (count) k_sort_keys<unsigned long long, true><<<grid, SORT_THREADS, 0, stream>>>(a, n, src_rows, tiles);
    else k_sort_keys<unsigned long long, false><<<grid, SORT_THREADS, 0, stream>>>(a, n, src_rows, tiles);
  }
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
  if ((kb != 4 && kb != 8) || shift >= kb * 8 || a.bytes[0] < n * kb || (uint64_t)tiles * RADIX * 4 > a.bytes[1] || a.bytes[2] < RADIX * 4)
    return (int)cudaErrorInvalidValue;
  uint32_t grid = cql_stream_grid(tiles, resident_ctas(kb == 4 ? (const void*)k_radix_count<uint32_t> : (const void*)k_radix_count<unsigned long long>, 0));
  if (kb == 4) k_radix_count<uint32_t><<<grid, SORT_THREADS, 0, stream>>>(a, n, tiles);
  else k_radix_count<unsigned long long><<<grid, SORT_THREADS, 0, stream>>>(a, n, tiles);
  CQL_LAUNCH_CHECK();
  return 0;
}

static int launch_radix_offsets(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t n = cql_word(a, 0);
  if (n == 0) return 0;
  uint32_t tiles = (uint32_t)((n + SORT_TILE - 1) / SORT_TILE);
  if ((uint64_t)tiles * RADIX * 4 > a.bytes[0] || a.bytes[1] < RADIX * 4 || (uint64_t)tiles * RADIX * 4 > a.bytes[2])
    return (int)cudaErrorInvalidValue;
  k_radix_offsets<<<RADIX, OFFSETS_THREADS, 0, stream>>>(a, tiles);
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
  if ((kb != 4 && kb != 8) || shift >= kb * 8 || a.bytes[0] < n * kb || (!cql_word(a, 10) && a.bytes[1] < n * 4) || a.bytes[3] < n * 4 ||
      (write_keys && a.bytes[2] < n * kb) || (uint64_t)tiles * RADIX * 4 > a.bytes[4] || (cql_word(a, 6) && a.bytes[5] < n * 4))
    return (int)cudaErrorInvalidValue;
  // the tile's keys and positions staged in dynamic shared memory
  size_t smem = (size_t)SORT_TILE * (kb + 4);
  const void* fn = kb == 4 ? (const void*)k_radix_scatter<uint32_t, SORT_RANK_FORM> : (const void*)k_radix_scatter<unsigned long long, SORT_RANK_FORM>;
  // dynamic plus static shared memory passes the default 48 KB for 8-byte keys: opt in
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  uint32_t grid = cql_stream_grid(tiles, resident_ctas(fn, smem));
  bool has_totals = a.buf[6] != nullptr && a.bytes[6] >= RADIX * 4;
  if (kb == 4) k_radix_scatter<uint32_t, SORT_RANK_FORM><<<grid, SORT_THREADS, smem, stream>>>(a, n, tiles, has_totals);
  else k_radix_scatter<unsigned long long, SORT_RANK_FORM><<<grid, SORT_THREADS, smem, stream>>>(a, n, tiles, has_totals);
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
  { "cql_radix_offsets", launch_radix_offsets },
  { "cql_radix_scatter", launch_radix_scatter },
  { nullptr, nullptr },
};
