// k_window.cu - ROW_NUMBER, RANK and DENSE_RANK over the rows in window order (the GPU window ranks of
// qe_window_rank_gpu, src/query_exec/query_exec.c:6155-6540, and window_rank_flags.comp), after the stable
// radix sort has put the rows in (partition keys, order keys) order.
//
//   cql_window_flags   per sorted position: does it start a partition (a partition key differs from the
//                      previous row's) and a peer group (any key differs); keys compared as F64 with !=, as
//                      window_rank_flags.comp compares them
//   cql_window_tiles   per tile of WIN_TILE positions: the tile's aggregate of the rank scan
//   cql_window_carry   one CTA: the exclusive scan of the tile aggregates
//   cql_window_apply   per tile: the scan within the tile from its carry, written out as the three ranks
//
// The scan element of position i is (last partition start, last peer start, any partition start, peer
// starts since the last partition start); combining (a then b) takes the larger positions and restarts
// the peer count where b holds a partition start. Then row_number = i - partition start + 1, rank = peer
// start - partition start + 1 and dense_rank = the peer count.
#include "cql_internal.cuh"

#define WIN_THREADS 256u
#define WIN_PER_THREAD 8u
#define WIN_TILE (WIN_THREADS * WIN_PER_THREAD)

struct WinAgg
{
  long long p, q;    // last partition start, last peer start (-1: none yet)
  unsigned h, d;     // a partition start inside; peer starts since the last partition start
};

__device__ __forceinline__ WinAgg win_identity()
{
  WinAgg r;
  r.p = -1;
  r.q = -1;
  r.h = 0u;
  r.d = 0u;
  return r;
}

__device__ __forceinline__ WinAgg win_combine(const WinAgg& a, const WinAgg& b)
{
  WinAgg r;
  r.p = a.p > b.p ? a.p : b.p;
  r.q = a.q > b.q ? a.q : b.q;
  r.h = a.h | b.h;
  r.d = b.h ? b.d : a.d + b.d;
  return r;
}

__device__ __forceinline__ WinAgg win_element(unsigned char flags, long long i)
{
  WinAgg r;
  r.p = (flags & 1u) ? i : -1;
  r.q = (flags & 2u) ? i : -1;
  r.h = flags & 1u;
  r.d = (flags >> 1) & 1u;
  return r;
}

__device__ __forceinline__ WinAgg win_shfl_up(const WinAgg& v, int o)
{
  WinAgg r;
  r.p = __shfl_up_sync(0xffffffffu, v.p, o);
  r.q = __shfl_up_sync(0xffffffffu, v.q, o);
  r.h = __shfl_up_sync(0xffffffffu, v.h, o);
  r.d = __shfl_up_sync(0xffffffffu, v.d, o);
  return r;
}

// Exclusive scan of one value per thread over the block; `total` receives the block's aggregate.
__device__ WinAgg win_block_exclusive(WinAgg v, WinAgg* total)
{
  __shared__ WinAgg s_warp[WIN_THREADS / 32];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  WinAgg incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    WinAgg y = win_shfl_up(incl, o);
    if (lane >= (unsigned)o) incl = win_combine(y, incl);
  }
  if (lane == 31u) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0)
  {
    WinAgg w = lane < WIN_THREADS / 32 ? s_warp[lane] : win_identity();
    WinAgg wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      WinAgg y = win_shfl_up(wi, o);
      if (lane >= (unsigned)o) wi = win_combine(y, wi);
    }
    if (lane < WIN_THREADS / 32) s_warp[lane] = wi;   // inclusive over warps
  }
  __syncthreads();
  WinAgg before_warp = warp ? s_warp[warp - 1] : win_identity();
  WinAgg lane_excl = win_shfl_up(incl, 1);
  if (lane == 0u) lane_excl = win_identity();
  *total = s_warp[WIN_THREADS / 32 - 1];
  WinAgg r = win_combine(before_warp, lane_excl);
  __syncthreads();
  return r;
}

// a key's value as the double the reference compares (64-bit integers rounded like the sort's keys)
__device__ __forceinline__ double win_key(const void* col, uint32_t type, uint32_t width, uint32_t base, uint64_t row)
{
  if (width == 3) return type == 7u ? (double)(int)(base + (uint32_t)row) : (double)(base + (uint32_t)row);
  if (width == 1 || width == 2)
  {
    uint32_t code = width == 1 ? ((const unsigned char*)col)[row] : ((const unsigned short*)col)[row];
    uint32_t v = base + code;
    return type == 7u || type == 9u ? (double)(int)v : (double)v;
  }
  switch (type)
  {
    case 1: case 12: return (double)((const uint32_t*)col)[row];
    case 7: case 9: return (double)((const int*)col)[row];
    case 3: return (double)((const float*)col)[row];
    case 2: case 10: return (double)((const unsigned long long*)col)[row];
    case 8: case 11: return (double)((const long long*)col)[row];
    default: return ((const double*)col)[row];
  }
}

// bindings 0 the sorted row numbers, 1 flags out (one byte per position), 2..5 the keys; words 0 n,
// 2 keys, 3 partition keys, 4 key types (8 bits each), 5 widths (8 bits each), 6..9 the keys' bases
__global__ void __launch_bounds__(WIN_THREADS) k_window_flags(CqlLaunch a, uint64_t n)
{
  const uint32_t* rows = (const uint32_t*)a.buf[0];
  unsigned char* flags = (unsigned char*)a.buf[1];
  const uint32_t nk = cql_word(a, 2), np = cql_word(a, 3), types = cql_word(a, 4), widths = cql_word(a, 5);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    if (i == 0)
    {
      flags[0] = 3u;
      continue;
    }
    const uint64_t r = rows[i], r0 = rows[i - 1];
    bool part = false, peer = false;
    for (uint32_t k = 0; k < nk && k < 4u; k++)
    {
      const uint32_t t = (types >> (8 * k)) & 0xffu, w = (widths >> (8 * k)) & 0xffu, base = cql_word(a, 6 + k);
      const double x = win_key(a.buf[2 + k], t, w, base, r), y = win_key(a.buf[2 + k], t, w, base, r0);
      if (x != y)
      {
        peer = true;
        if (k < np) part = true;
      }
    }
    flags[i] = (part ? 1u : 0u) | (peer || part ? 2u : 0u);
  }
}

static int launch_window_flags(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t n = cql_word(a, 0);
  if (n == 0) return 0;
  if (a.bytes[0] < n * 4 || a.bytes[1] < n) return (int)cudaErrorInvalidValue;
  k_window_flags<<<cql_stream_grid((n + WIN_THREADS - 1) / WIN_THREADS, 8), WIN_THREADS, 0, stream>>>(a, n);
  CQL_LAUNCH_CHECK();
  return 0;
}

// the scan of one tile from `carry`: per position the running element; `emit` writes the ranks
template <bool EMIT>
__device__ WinAgg win_tile(const unsigned char* flags, uint64_t n, uint64_t tile, WinAgg carry, uint32_t* row_number, uint32_t* rank,
                           uint32_t* dense)
{
  const uint64_t first = tile * WIN_TILE + (uint64_t)threadIdx.x * WIN_PER_THREAD;
  unsigned char f[WIN_PER_THREAD];
#pragma unroll
  for (uint32_t j = 0; j < WIN_PER_THREAD; j++) f[j] = first + j < n ? flags[first + j] : 0u;
  WinAgg mine = win_identity();
#pragma unroll
  for (uint32_t j = 0; j < WIN_PER_THREAD; j++)
    if (first + j < n) mine = win_combine(mine, win_element(f[j], (long long)(first + j)));
  WinAgg total;
  WinAgg run = win_combine(carry, win_block_exclusive(mine, &total));
  if (EMIT)
  {
#pragma unroll
    for (uint32_t j = 0; j < WIN_PER_THREAD; j++)
    {
      const uint64_t i = first + j;
      if (i >= n) break;
      run = win_combine(run, win_element(f[j], (long long)i));
      row_number[i] = (uint32_t)((long long)i - run.p + 1);
      rank[i] = (uint32_t)(run.q - run.p + 1);
      dense[i] = run.d;
    }
  }
  return total;
}

// bindings 0 flags, 1 the tile aggregates out; word 0 n
__global__ void __launch_bounds__(WIN_THREADS) k_window_tiles(CqlLaunch a, uint64_t n, uint64_t tiles)
{
  const unsigned char* flags = (const unsigned char*)a.buf[0];
  WinAgg* agg = (WinAgg*)a.buf[1];
  for (uint64_t t = blockIdx.x; t < tiles; t += gridDim.x)
  {
    WinAgg total = win_tile<false>(flags, n, t, win_identity(), nullptr, nullptr, nullptr);
    if (threadIdx.x == 0) agg[t] = total;
  }
}

static int launch_window_tiles(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t n = cql_word(a, 0);
  if (n == 0) return 0;
  uint64_t tiles = (n + WIN_TILE - 1) / WIN_TILE;
  if (a.bytes[0] < n || a.bytes[1] < tiles * sizeof(WinAgg)) return (int)cudaErrorInvalidValue;
  k_window_tiles<<<cql_stream_grid(tiles, 8), WIN_THREADS, 0, stream>>>(a, n, tiles);
  CQL_LAUNCH_CHECK();
  return 0;
}

// bindings 0 the tile aggregates, 1 the carries out (exclusive); word 0 tiles
__global__ void __launch_bounds__(WIN_THREADS) k_window_carry(CqlLaunch a, uint64_t tiles)
{
  const WinAgg* agg = (const WinAgg*)a.buf[0];
  WinAgg* carry = (WinAgg*)a.buf[1];
  WinAgg run = win_identity();
  for (uint64_t base = 0; base < tiles; base += WIN_THREADS)
  {
    const uint64_t t = base + threadIdx.x;
    WinAgg v = t < tiles ? agg[t] : win_identity();
    WinAgg total;
    WinAgg excl = win_block_exclusive(v, &total);
    if (t < tiles) carry[t] = win_combine(run, excl);
    run = win_combine(run, total);
  }
}

static int launch_window_carry(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t tiles = cql_word(a, 0);
  if (tiles == 0) return 0;
  if (a.bytes[0] < tiles * sizeof(WinAgg) || a.bytes[1] < tiles * sizeof(WinAgg)) return (int)cudaErrorInvalidValue;
  k_window_carry<<<1, WIN_THREADS, 0, stream>>>(a, tiles);
  CQL_LAUNCH_CHECK();
  return 0;
}

// bindings 0 flags, 1 the carries, 2 row_number, 3 rank, 4 dense_rank (u32 per position); word 0 n
__global__ void __launch_bounds__(WIN_THREADS) k_window_apply(CqlLaunch a, uint64_t n, uint64_t tiles)
{
  const unsigned char* flags = (const unsigned char*)a.buf[0];
  const WinAgg* carry = (const WinAgg*)a.buf[1];
  uint32_t* row_number = (uint32_t*)a.buf[2];
  uint32_t* rank = (uint32_t*)a.buf[3];
  uint32_t* dense = (uint32_t*)a.buf[4];
  for (uint64_t t = blockIdx.x; t < tiles; t += gridDim.x) win_tile<true>(flags, n, t, carry[t], row_number, rank, dense);
}

static int launch_window_apply(const CqlLaunch& a, uint32_t gws, uint32_t lws, cudaStream_t stream)
{
  (void)gws;
  (void)lws;
  uint64_t n = cql_word(a, 0);
  if (n == 0) return 0;
  uint64_t tiles = (n + WIN_TILE - 1) / WIN_TILE;
  if (a.bytes[0] < n || a.bytes[1] < tiles * sizeof(WinAgg) || a.bytes[2] < n * 4 || a.bytes[3] < n * 4 || a.bytes[4] < n * 4)
    return (int)cudaErrorInvalidValue;
  k_window_apply<<<cql_stream_grid(tiles, 8), WIN_THREADS, 0, stream>>>(a, n, tiles);
  CQL_LAUNCH_CHECK();
  return 0;
}

const CqlKernelDesc cql_kernels_window[] = {
  { "cql_window_flags", launch_window_flags },
  { "cql_window_tiles", launch_window_tiles },
  { "cql_window_carry", launch_window_carry },
  { "cql_window_apply", launch_window_apply },
  { nullptr, nullptr },
};
