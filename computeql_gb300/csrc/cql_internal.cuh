// Internal interface between the runtime (runtime.cu) and the kernel families (k_*.cu).
//
// A reference kernel is dispatched with a binding table and eight U64 push-constant slots
// (src/gpu/vulkan/gpu_vulkan.h:6-9). The runtime packs them into CqlLaunch, passes it by value,
// and the kernel reads slot words exactly as the shader reads pc.words[] (low word first).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define CQL_MAX_BINDINGS 16
#define CQL_PUSH_SLOTS   8

struct CqlLaunch
{
  void* buf[CQL_MAX_BINDINGS];
  uint64_t bytes[CQL_MAX_BINDINGS];   // bound range of each binding, what `.length()` sees in the shader
  uint64_t push[CQL_PUSH_SLOTS];
};

// pc.words[i] of the shader: the low (even i) or high (odd i) half of slot i/2.
__host__ __device__ inline uint32_t cql_word(const CqlLaunch& a, uint32_t i)
{
  uint64_t slot = a.push[i >> 1];
  return (i & 1u) ? (uint32_t)(slot >> 32) : (uint32_t)slot;
}

// A launcher decodes the contract, picks its own grid and enqueues on `stream`.
// Returns 0 on success, a cudaError_t otherwise. `gws`/`lws` are what the caller asked for.
typedef int (*CqlLauncher)(const CqlLaunch& args, uint32_t gws, uint32_t lws, cudaStream_t stream);

struct CqlKernelDesc
{
  const char* name;
  CqlLauncher launch;
};

// Each k_*.cu file exports a table of its kernels; the runtime concatenates them.
extern const CqlKernelDesc cql_kernels_aggregate[];
extern const CqlKernelDesc cql_kernels_scan[];
extern const CqlKernelDesc cql_kernels_hash[];
extern const CqlKernelDesc cql_kernels_join[];
extern const CqlKernelDesc cql_kernels_sort[];
extern const CqlKernelDesc cql_kernels_fixed[];
extern const CqlKernelDesc cql_kernels_window[];

// Device facts the launchers size grids by (set once by cqlcuda_init).
extern int g_cql_sm_count;
extern int g_cql_max_smem_optin;

// Counts launches of this library's kernels (the figure a bench reports as gpu_launches).
void cql_note_launch(void);

// Sets the calling thread's cqlcuda_last_error() text (printf format).
void cql_set_error_text(const char* fmt, ...);

// Resolves the no-allocation slot compaction's static scratch for the current device and loads its
// kernel, so that the entry point's later calls allocate nothing even under lazy module loading.
// Returns 1 on success. cqlcuda_init calls it for the device it opens.
int cql_noalloc_prepare(void);

#define CQL_LAUNCH_CHECK() do { cudaError_t e__ = cudaGetLastError(); if (e__ != cudaSuccess) return (int)e__; cql_note_launch(); } while (0)

// Grid for a streaming kernel: `per_sm` resident CTAs on every SM, never more CTAs than `work_ctas`.
static inline uint32_t cql_stream_grid(uint64_t work_ctas, int per_sm)
{
  uint64_t g = (uint64_t)g_cql_sm_count * (uint64_t)per_sm;
  if (work_ctas < g) g = work_ctas;
  if (g == 0) g = 1;
  return (uint32_t)g;
}

// A full-width numeric value as the f64 the reference widens it to on the host (query_exec.c:10454-10690):
// type is the CQL column type (1 U32, 2 U64, 3 F32, 4 F64, 7 I32, 8 I64).
__device__ __forceinline__ double cql_value_as_f64(const void* p, uint32_t type, uint64_t row)
{
  switch (type)
  {
    case 1: return (double)((const uint32_t*)p)[row];
    case 7: return (double)((const int*)p)[row];
    case 3: return (double)__uint_as_float(((const uint32_t*)p)[row]);
    case 2: return (double)((const unsigned long long*)p)[row];
    case 8: return (double)((const long long*)p)[row];
    default: return ((const double*)p)[row];
  }
}

// Order-preserving maps used by kernels that keep f64 min/max in integer registers.
__device__ __forceinline__ unsigned long long cql_f64_order_key(double x)
{
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double cql_f64_from_order_key(unsigned long long k)
{
  unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}
