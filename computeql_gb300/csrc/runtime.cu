// GB300 runtime behind the cqlcuda C ABI: device, buffers, pooled buffers with epochs and
// eviction, host import, kernels by shader name, NVRTC-built kernels, batches, multi-slot
// streams, kernel profile, failure injection.
//
// It replaces the Vulkan backend (src/gpu/vulkan/gpu_vulkan.c) behind the same vtable
// (src/gpu/gpu_backend.h:17-71). Design differences, GB300-first:
//  - device memory is plain cudaMalloc, one allocation per buffer (no sub-allocated blocks, no
//    ReBAR heap): 280 GB of HBM makes block sub-allocation unnecessary;
//  - a batch is the runtime's stream plus a pinned staging area for reads, finished by one
//    bounded synchronise (gpu_vulkan.c:2864-3116 records a command buffer and waits on a fence);
//  - each stream slot is a CUDA stream with its own pinned readback staging; submit records an
//    event, wait polls it with a time limit instead of aborting (gpu_vulkan.c:1106-1135, 1390-1480);
//  - kernel time comes from CUDA event pairs (gpu_vulkan.c:2976-2993 uses timestamp queries).
#include "cql_internal.cuh"
#include <atomic>
#include "../../include/cqlcuda.h"

#include <nvrtc.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <shared_mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>
#include <sys/mman.h>
#include <sys/syscall.h>
#include <unistd.h>

int g_cql_sm_count = 152;
int g_cql_max_smem_optin = 227 * 1024;

// ---------------------------------------------------------------------------------------------
// state

struct CqlBuffer
{
  void* dptr;
  uint64_t size;       // bound range seen by kernels
  uint64_t capacity;   // bytes allocated
  uint32_t flags;
  int imported;        // host memory registered (or directly addressable), not owned
  const void* host_ptr;
  uint64_t charge;     // device bytes charged to the memory stats
};

struct CqlPooled
{
  std::string name;
  CqlBuffer* buffer;
  uint64_t capacity;
  uint64_t last_epoch;
  const void* imported_host_ptr;
};

struct CqlKernel
{
  std::string name;
  CqlLauncher builtin;        // precompiled kernel family
  cudaKernel_t generated;     // NVRTC-built kernel, launched with CqlLaunch by value
  cudaLibrary_t library;      // the module a generated kernel lives in (unloaded when it is evicted)
  uint64_t last_use;          // tick of its last lookup, for the generated-kernel cap
  uint32_t gen_block;         // block size a generated kernel declares (256 unless its source says otherwise)
  uint32_t gen_smem;          // dynamic shared memory a generated kernel asks for
  uint32_t gen_per_sm;        // resident CTAs per SM the grid is sized for
  CqlLaunch args;
  uint32_t spec[16];
  uint32_t spec_count;
  uint32_t profile_index;
};

struct CqlPendingRead
{
  void* dst;
  uint64_t staging_offset;
  uint64_t size;
};

struct CqlTiming
{
  uint32_t profile_index;
  cudaEvent_t start;
  cudaEvent_t stop;
};

struct CqlStaging
{
  unsigned char* host;   // pinned
  uint64_t capacity;
  uint64_t used;
  std::vector<CqlPendingRead> reads;
};

// A batch opened for a plan shape (cqlcuda_batch_begin_graph) records its operations instead of issuing
// them; at its end the record's fingerprint (every operation, buffer address, size and kernel argument,
// not the bytes written) finds the CUDA graph captured for that shape, which is replayed with the new
// bytes, or the record is captured into a new graph.
enum
{
  CQL_OP_WRITE,
  CQL_OP_ZERO,
  CQL_OP_FILL,
  CQL_OP_KERNEL,
  CQL_OP_READ,
};

struct CqlOp
{
  int kind;
  CqlBuffer* buffer;
  void* dptr;         // the buffer's device address when recorded: a captured graph's entry keeps it, since
                      // the CqlBuffer itself may be freed while the graph stays cached
  uint64_t offset, size;
  uint32_t value;
  uint64_t at;        // WRITE: the bytes' place in the record; READ: the result's place in the out area
  void* out;          // READ: the caller's destination
  CqlKernel* kernel;  // KERNEL: with its arguments as they were when it was recorded
  CqlLaunch launch;
  uint32_t gws, lws;
};

struct CqlGraphEntry
{
  cudaGraphExec_t exec;
  unsigned char* in;    // pinned: the bytes the graph uploads
  unsigned char* out;   // pinned: the results it downloads
  uint64_t in_size, out_size;
  uint32_t kernels;
  uint64_t last_use;
  uint64_t plan_key;
  std::vector<CqlOp> ops;   // the record it was captured from: a fingerprint hit must equal it
};

struct CqlBatch
{
  int active;
  int failed;
  std::chrono::steady_clock::time_point opened;   // for the host-side entries of the kernel profile
  CqlStaging staging;
  int recording;
  uint64_t plan_key;
  std::vector<CqlOp> ops;
  std::vector<unsigned char> in_bytes;
  uint64_t out_bytes;
};

struct CqlStreamSlot
{
  cudaStream_t stream;
  cudaEvent_t done;
  int submitted;
  int failed;
  CqlStaging staging;
  std::vector<CqlTiming> timings;
};

struct CqlStream
{
  uint32_t slot_count;
  CqlStreamSlot slots[8];
  CqlStreamStats stats;
};

struct CqlProfileEntry
{
  std::string name;
  uint64_t total_ns;
  uint64_t dispatches;
};

// A lane is where a thread's batches run: a stream, a batch with its staging area and timings, the
// kernel arguments the thread has set, and the tag its pooled buffers are named under. The process
// has one main lane (the reference's single queue: one batch at a time); a thread that opens its own
// lane (cqlcuda_thread_lane_begin) runs its batches on its own stream, concurrently with the others.
struct CqlLane
{
  cudaStream_t stream;
  CqlBatch batch;
  std::vector<CqlTiming> timings;
  std::string pool_tag;
  std::unordered_map<const CqlKernel*, CqlLaunch> args;
  uint32_t launches;     // kernels this lane launched
  int is_main;
  std::unordered_map<uint64_t, CqlGraphEntry> graphs;   // plan graphs by fingerprint, this lane's alone
  uint64_t graph_clock;
  std::unordered_map<uint64_t, uint32_t> graph_seen;    // fingerprints met once: captured when met again
};

static std::atomic<uint64_t> g_graph_captures{0}, g_graph_replays{0}, g_graph_fallbacks{0};
static std::atomic<int> g_graphs_on{1};

struct CqlState
{
  int initialized;
  int device;
  int device_lost;
  cudaStream_t stream;
  cudaEvent_t exec_start, exec_stop, timer_start, timer_stop;
  int pageable_access;

  CqlMemoryStats mem;
  uint64_t pool_epoch;
  std::vector<CqlPooled> pool;
  std::unordered_map<std::string, size_t> pool_index;
  CqlEvictHook evict_hook;
  uint64_t fault_alloc_at;

  std::unordered_map<std::string, CqlKernel*> kernels;
  uint64_t generated_compiles;
  uint64_t generated_evictions;
  uint32_t generated_cap;                // generated kernels kept loaded (GPU_VULKAN_MAX_GENERATED_KERNELS)
  uint64_t kernel_tick;
  std::vector<CqlKernel*> retired;       // evicted kernels: their objects stay valid, their modules are gone
  std::string cache_dir;
  uint32_t fail_compile_every;
  uint64_t compile_attempts;
  std::string compile_log;

  CqlLane main_lane;
  uint32_t lanes_open;   // threads with a lane of their own (pool eviction waits until they close)
  uint32_t persistent_open;   // persistent kernels created and not destroyed (no generated kernel is evicted meanwhile)

  int profile_enabled;
  std::atomic<uint64_t> host_open_ns, host_wait_ns, host_copy_ns, host_batches;
  std::vector<CqlProfileEntry> profile;
  std::unordered_map<std::string, uint32_t> profile_index;

  uint64_t last_kernel_us;
  std::atomic<uint32_t> launches;
  uint32_t wait_timeout_ms;

  void* flush_buf;
  uint64_t flush_bytes;

  std::recursive_mutex lock;
  std::shared_mutex generated_use;   // launches of generated kernels (shared) against their eviction (exclusive)
};

// Generated kernels kept loaded, as the reference's GPU_VULKAN_MAX_GENERATED_KERNELS (default 64, at least
// 8, src/gpu/vulkan/gpu_vulkan.c:75); the least recently looked-up one is evicted past the cap
// (:2721-2737). The 8 most recently looked-up kernels are never evicted: an operator looks up the few
// kernels it launches just before it launches them.
#define CQL_GENERATED_KERNEL_CAP 64
#define CQL_GENERATED_KERNEL_MIN_CAP 8

static CqlState* g_state = nullptr;

static CqlState& S()
{
  if (!g_state)
  {
    g_state = new CqlState();
    g_state->initialized = 0;
    g_state->device_lost = 0;
    g_state->pool_epoch = 1;
    g_state->evict_hook = nullptr;
    g_state->fault_alloc_at = 0;
    g_state->generated_compiles = 0;
    g_state->generated_evictions = 0;
    g_state->generated_cap = CQL_GENERATED_KERNEL_CAP;
    g_state->kernel_tick = 0;
    g_state->fail_compile_every = 0;
    g_state->compile_attempts = 0;
    g_state->profile_enabled = 0;
    g_state->host_batches = 0;
    g_state->host_open_ns = 0;
    g_state->host_wait_ns = 0;
    g_state->host_copy_ns = 0;
    g_state->last_kernel_us = 0;
    g_state->launches = 0;
    g_state->wait_timeout_ms = 30000;
    g_state->flush_buf = nullptr;
    g_state->flush_bytes = 0;
    memset(&g_state->mem, 0, sizeof(g_state->mem));
    CqlLane& m = g_state->main_lane;
    m.stream = nullptr;
    m.batch.active = 0;
    m.batch.failed = 0;
    m.batch.staging.host = nullptr;
    m.batch.staging.capacity = 0;
    m.batch.staging.used = 0;
    m.is_main = 1;
    m.launches = 0;
    g_state->lanes_open = 0;
    g_state->persistent_open = 0;
  }
  return *g_state;
}

static thread_local CqlLane* tl_lane = nullptr;
static thread_local std::string tl_error;

// the calling thread's lane
static CqlLane& L() { return tl_lane ? *tl_lane : S().main_lane; }

void cql_note_launch(void)
{
  S().launches.fetch_add(1, std::memory_order_relaxed);
  if (tl_lane) tl_lane->launches += 1;
}

static void set_error(const char* fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  tl_error = buf;
}

void cql_set_error_text(const char* fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  tl_error = buf;
}

// A CUDA error that leaves the context unusable makes device_lost sticky, as
// gpu_vulkan_note_result does for VK_ERROR_DEVICE_LOST (gpu_vulkan.c:1523-1535).
static int note_cuda(cudaError_t e, const char* what)
{
  if (e == cudaSuccess) return 1;
  set_error("%s: %s (%d)", what, cudaGetErrorString(e), (int)e);
  switch (e)
  {
    case cudaErrorIllegalAddress:
    case cudaErrorLaunchFailure:
    case cudaErrorIllegalInstruction:
    case cudaErrorMisalignedAddress:
    case cudaErrorInvalidAddressSpace:
    case cudaErrorInvalidPc:
    case cudaErrorHardwareStackError:
    case cudaErrorAssert:
    case cudaErrorLaunchTimeout:
    case cudaErrorECCUncorrectable:
      S().device_lost = 1;
      break;
    default:
      break;
  }
  return 0;
}

// Bounded wait on a stream: polls until done or the wait limit, never blocks forever.
// Waits poll without sleeping for the first CQL_SPIN_US microseconds, so that a short query's result is
// seen within microseconds of the GPU finishing (a sleep on Linux overshoots by tens of microseconds,
// which short queries would pay at every wait). Between polls the thread waits on the clock, about 1 % of
// the time waited so far (1 to 20 us), without calling the driver: polling it back to back slowed
// host-to-device copies in flight by a third. Longer waits sleep 20 us between polls. Every wait ends
// with an error after the wait timeout instead of blocking for ever.
#define CQL_SPIN_US 20000

template <typename Query>
static int wait_polled(Query done, const char* what)
{
  auto t0 = std::chrono::steady_clock::now();
  for (;;)
  {
    cudaError_t e = done();
    if (e == cudaSuccess) return 1;
    if (e != cudaErrorNotReady) return note_cuda(e, what);
    auto now = std::chrono::steady_clock::now();
    auto us = std::chrono::duration_cast<std::chrono::microseconds>(now - t0).count();
    if ((uint64_t)us > (uint64_t)S().wait_timeout_ms * 1000ull)
    {
      set_error("%s: GPU work did not complete within %u ms", what, S().wait_timeout_ms);
      return 0;
    }
    if (us > CQL_SPIN_US)
    {
      std::this_thread::sleep_for(std::chrono::microseconds(20));
      continue;
    }
    auto gap = std::chrono::microseconds(1 + std::min<long long>(19, (long long)us / 100));
    while (std::chrono::steady_clock::now() - now < gap)
    {
    }
  }
}

static int wait_stream(cudaStream_t stream, const char* what)
{
  return wait_polled([stream]() { return cudaStreamQuery(stream); }, what);
}

static int wait_event(cudaEvent_t ev, const char* what)
{
  return wait_polled([ev]() { return cudaEventQuery(ev); }, what);
}

// ---------------------------------------------------------------------------------------------
// profile

static uint32_t profile_slot(const std::string& name)
{
  CqlState& s = S();
  auto it = s.profile_index.find(name);
  if (it != s.profile_index.end()) return it->second;
  uint32_t idx = (uint32_t)s.profile.size();
  s.profile.push_back(CqlProfileEntry{name, 0, 0});
  s.profile_index[name] = idx;
  return idx;
}

// Timing events are reused: creating and destroying two events per dispatch would cost the profiled
// run microseconds per kernel.
static std::mutex g_event_pool_lock;
static std::vector<cudaEvent_t> g_event_pool;

static cudaEvent_t timing_event_get()
{
  {
    std::lock_guard<std::mutex> g(g_event_pool_lock);
    if (!g_event_pool.empty())
    {
      cudaEvent_t e = g_event_pool.back();
      g_event_pool.pop_back();
      return e;
    }
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

static void timing_event_put(cudaEvent_t e)
{
  if (!e) return;
  std::lock_guard<std::mutex> g(g_event_pool_lock);
  g_event_pool.push_back(e);
}

static void timings_collect(std::vector<CqlTiming>& timings)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  for (auto& t : timings)
  {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, t.start, t.stop) == cudaSuccess)
    {
      s.profile[t.profile_index].total_ns += (uint64_t)((double)ms * 1e6);
      s.profile[t.profile_index].dispatches += 1;
      s.last_kernel_us = (uint64_t)((double)ms * 1e3);
    }
    timing_event_put(t.start);
    timing_event_put(t.stop);
  }
  timings.clear();
}

// ---------------------------------------------------------------------------------------------
// device

extern "C" int cqlcuda_init(void)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  if (s.initialized) return !s.device_lost;
  int count = 0;
  if (!note_cuda(cudaGetDeviceCount(&count), "cudaGetDeviceCount")) return 0;
  if (count <= 0)
  {
    set_error("cqlcuda_init: no CUDA device");
    return 0;
  }
  s.device = 0;
  if (!note_cuda(cudaSetDevice(s.device), "cudaSetDevice")) return 0;
  cudaDeviceProp prop;
  if (!note_cuda(cudaGetDeviceProperties(&prop, s.device), "cudaGetDeviceProperties")) return 0;
  if (prop.major < 10)
  {
    set_error("cqlcuda_init: device %s is sm_%d%d, this library is built for sm_103a", prop.name, prop.major, prop.minor);
    return 0;
  }
  g_cql_sm_count = prop.multiProcessorCount;
  g_cql_max_smem_optin = (int)prop.sharedMemPerBlockOptin;
  int pageable = 0;
  cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, s.device);
  s.pageable_access = pageable;
  if (!note_cuda(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "cudaStreamCreate")) return 0;
  s.main_lane.stream = s.stream;
  cudaEventCreate(&s.exec_start);
  cudaEventCreate(&s.exec_stop);
  cudaEventCreate(&s.timer_start);
  cudaEventCreate(&s.timer_stop);
  // the no-allocation compaction's scratch address and kernel, resolved now rather than mid-query
  cql_noalloc_prepare();
  s.initialized = 1;
  return 1;
}

static int ensure_init(void)
{
  if (S().initialized) return !S().device_lost;
  return cqlcuda_init();
}

static void staging_release(CqlStaging& st)
{
  if (st.host) cudaFreeHost(st.host);
  st.host = nullptr;
  st.capacity = 0;
  st.used = 0;
  st.reads.clear();
}

extern "C" void cqlcuda_release(void)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  if (!s.initialized) return;
  cudaStreamSynchronize(s.stream);
  for (auto& p : s.pool)
  {
    if (p.buffer) cqlcuda_buffer_release(p.buffer);
    p.buffer = nullptr;
  }
  s.pool.clear();
  s.pool_index.clear();
  for (auto& kv : s.kernels)
  {
    if (kv.second->library) cudaLibraryUnload(kv.second->library);
    delete kv.second;
  }
  for (CqlKernel* k : s.retired) delete k;
  s.retired.clear();
  s.kernels.clear();
  staging_release(s.main_lane.batch.staging);
  if (s.flush_buf) cudaFree(s.flush_buf);
  s.flush_buf = nullptr;
  cudaStreamDestroy(s.stream);
  s.initialized = 0;
}

extern "C" void cqlcuda_wait(void)
{
  if (!S().initialized) return;
  wait_stream(L().stream ? L().stream : S().stream, "cqlcuda_wait");
}

extern "C" uint64_t cqlcuda_get_executed_kernel_time_microseconds(void) { return S().last_kernel_us; }

extern "C" uint64_t cqlcuda_device_total_memory(void)
{
  if (!ensure_init()) return 0;
  size_t f = 0, t = 0;
  cudaMemGetInfo(&f, &t);
  return t;
}

extern "C" uint64_t cqlcuda_device_free_memory(void)
{
  if (!ensure_init()) return 0;
  size_t f = 0, t = 0;
  cudaMemGetInfo(&f, &t);
  return f;
}

// No binding-range limit applies to a CUDA pointer; report the device memory so the operator
// layer's GPU_MAX_BUFFER_SIZE-style chunking (src/main.c:7) never has to split a resident column.
extern "C" uint64_t cqlcuda_device_max_storage_buffer_range(void) { return cqlcuda_device_total_memory(); }
extern "C" int cqlcuda_device_lost(void) { return S().device_lost; }
extern "C" void cqlcuda_pool_begin_epoch(void) { S().pool_epoch += 1; }
extern "C" CqlMemoryStats cqlcuda_memory_stats(void) { return S().mem; }
extern "C" uint32_t cqlcuda_sm_count(void) { ensure_init(); return (uint32_t)g_cql_sm_count; }

// ---------------------------------------------------------------------------------------------
// buffers

// Pooled buffers no running query looked up in this epoch are freed, oldest first
// (gpu_vulkan_pool_evict, gpu_vulkan.c:1577-1617).
static uint64_t pool_evict(uint64_t bytes_wanted)
{
  CqlState& s = S();
  // never while a batch is recording: its buffers are bound (any lane's batch)
  if (s.main_lane.batch.active || s.lanes_open) return 0;
  uint64_t freed = 0;
  while (freed < bytes_wanted)
  {
    CqlPooled* victim = nullptr;
    for (auto& p : s.pool)
    {
      if (!p.buffer || p.buffer->charge == 0 || p.last_epoch >= s.pool_epoch) continue;
      if (!victim || p.last_epoch < victim->last_epoch) victim = &p;
    }
    if (!victim) break;
    uint64_t charge = victim->buffer->charge;
    cqlcuda_buffer_release(victim->buffer);
    victim->buffer = nullptr;
    victim->capacity = 0;
    victim->imported_host_ptr = nullptr;
    freed += charge;
    s.mem.pool_evictions += 1;
    s.mem.pool_evicted_bytes += charge;
  }
  return freed;
}

extern "C" uint64_t cqlcuda_pool_evict(uint64_t bytes_wanted)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  if (!s.initialized) return 0;
  cudaStreamSynchronize(s.stream);
  return pool_evict(bytes_wanted);
}

// The k-th allocation call fails when fault_alloc_at == k (gpu_vulkan_fault_injected, gpu_vulkan.c:1619-1631).
static int fault_injected(const char* what, uint64_t size)
{
  CqlState& s = S();
  s.mem.alloc_calls += 1;
  if (s.fault_alloc_at == 0 || s.mem.alloc_calls != s.fault_alloc_at) return 0;
  s.mem.alloc_failures += 1;
  set_error("cqlcuda: injected failure of allocation %llu (%s, %llu bytes)", (unsigned long long)s.mem.alloc_calls, what,
            (unsigned long long)size);
  return 1;
}

static void* device_alloc(uint64_t size)
{
  CqlState& s = S();
  void* p = nullptr;
  uint64_t bytes = size ? size : 16;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e == cudaErrorMemoryAllocation)
  {
    cudaGetLastError();
    uint64_t freed = pool_evict(bytes);
    if (freed < bytes && s.evict_hook) freed += s.evict_hook(bytes - freed);
    if (freed > 0)
    {
      e = cudaMalloc(&p, bytes);
      if (e == cudaSuccess) s.mem.alloc_retry_successes += 1;
      else cudaGetLastError();
    }
  }
  if (e != cudaSuccess)
  {
    s.mem.alloc_failures += 1;
    s.mem.unrecovered_alloc_failures += 1;
    set_error("cqlcuda: cudaMalloc of %llu bytes failed: %s", (unsigned long long)bytes, cudaGetErrorString(e));
    return nullptr;
  }
  s.mem.bytes_in_use += bytes;
  s.mem.bytes_peak = std::max(s.mem.bytes_peak, s.mem.bytes_in_use);
  return p;
}

extern "C" CqlBuffer* cqlcuda_buffer_alloc(uint64_t size, uint32_t flags, const void* data)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  if (!ensure_init()) return nullptr;
  if (fault_injected("buffer", size)) return nullptr;
  void* p = device_alloc(size);
  if (!p) return nullptr;
  CqlBuffer* b = new CqlBuffer();
  b->dptr = p;
  b->size = size;
  b->capacity = size ? size : 16;
  b->flags = flags;
  b->imported = 0;
  b->host_ptr = nullptr;
  b->charge = b->capacity;
  if (data && size)
  {
    if (!note_cuda(cudaMemcpyAsync(p, data, size, cudaMemcpyHostToDevice, s.stream), "buffer_alloc upload") ||
        !wait_stream(s.stream, "buffer_alloc upload"))
    {
      cqlcuda_buffer_release(b);
      return nullptr;
    }
  }
  return b;
}

static CqlPooled* pool_find(const std::string& name)
{
  auto it = S().pool_index.find(name);
  return it == S().pool_index.end() ? nullptr : &S().pool[it->second];
}

// Reused while its capacity covers the request; a bigger request replaces it
// (gpu_vulkan_buffer_alloc_pooled, gpu_vulkan.c:2167-2211).
extern "C" CqlBuffer* cqlcuda_buffer_alloc_pooled(const char* name, uint64_t name_len, uint64_t size, uint32_t flags, const void* data)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  std::string key = L().pool_tag + std::string(name, name_len);
  CqlPooled* slot = pool_find(key);
  if (slot)
  {
    slot->last_epoch = s.pool_epoch;
    if (size > slot->capacity || !slot->buffer || slot->imported_host_ptr)
    {
      cqlcuda_buffer_release(slot->buffer);
      slot->buffer = cqlcuda_buffer_alloc(size, flags, data);
      slot->capacity = slot->buffer ? size : 0;
      slot->imported_host_ptr = nullptr;
    }
    else
    {
      slot->buffer->size = size;
      if (data) cqlcuda_buffer_write(slot->buffer, data, size);
    }
    return slot->buffer;
  }
  CqlBuffer* b = cqlcuda_buffer_alloc(size, flags, data);
  s.pool.push_back(CqlPooled{key, b, b ? size : 0, s.pool_epoch, nullptr});
  s.pool_index[key] = s.pool.size() - 1;
  return b;
}

// Host memory is pinned and mapped read-only; on a GB300 node (NVLink-C2C, ATS) the GPU could also
// read pageable memory directly, which is the fallback when registration is refused.
extern "C" CqlBuffer* cqlcuda_buffer_import_host_readonly(const void* host_ptr, uint64_t size)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  if (!ensure_init() || !host_ptr || size == 0) return nullptr;
  if (fault_injected("import", size)) return nullptr;
  void* dptr = nullptr;
  int registered = 0;
  cudaError_t e = cudaHostRegister(const_cast<void*>(host_ptr), size, cudaHostRegisterMapped | cudaHostRegisterReadOnly);
  if (e == cudaSuccess)
  {
    registered = 1;
    if (cudaHostGetDevicePointer(&dptr, const_cast<void*>(host_ptr), 0) != cudaSuccess)
    {
      cudaHostUnregister(const_cast<void*>(host_ptr));
      registered = 0;
      dptr = nullptr;
    }
  }
  else
  {
    cudaGetLastError();
  }
  if (!dptr && s.pageable_access) dptr = const_cast<void*>(host_ptr);
  if (!dptr)
  {
    set_error("cqlcuda_buffer_import_host_readonly: host memory at %p (%llu bytes) cannot be mapped", host_ptr, (unsigned long long)size);
    return nullptr;
  }
  CqlBuffer* b = new CqlBuffer();
  b->dptr = dptr;
  b->size = size;
  b->capacity = size;
  b->flags = CQLCUDA_BUFFER_READ;
  b->imported = registered ? 1 : 2;
  b->host_ptr = host_ptr;
  b->charge = 0;
  return b;
}

// page-locked host memory mapped into the device's address space, owned by the buffer: kernels write results
// there that the host reads without a copy (a persistent kernel's answers)
extern "C" CqlBuffer* cqlcuda_buffer_alloc_host_mapped(uint64_t size, void** out_host)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  if (out_host) *out_host = nullptr;
  if (!ensure_init() || size == 0) return nullptr;
  if (fault_injected("host_mapped", size)) return nullptr;
  void* h = nullptr;
  void* d = nullptr;
  if (!note_cuda(cudaHostAlloc(&h, size, cudaHostAllocMapped), "cudaHostAlloc(mapped)")) return nullptr;
  memset(h, 0, size);
  if (!note_cuda(cudaHostGetDevicePointer(&d, h, 0), "cudaHostGetDevicePointer"))
  {
    cudaFreeHost(h);
    return nullptr;
  }
  CqlBuffer* b = new CqlBuffer();
  b->dptr = d;
  b->size = size;
  b->capacity = size;
  b->flags = CQLCUDA_BUFFER_READ_WRITE;
  b->imported = 3;
  b->host_ptr = h;
  b->charge = 0;
  if (out_host) *out_host = h;
  return b;
}

extern "C" CqlBuffer* cqlcuda_buffer_import_host_readonly_pooled(const char* name, uint64_t name_len, const void* host_ptr, uint64_t size)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  std::string key = L().pool_tag + std::string(name, name_len);
  CqlPooled* slot = pool_find(key);
  if (slot && slot->buffer && slot->imported_host_ptr == host_ptr && slot->capacity == size)
  {
    slot->last_epoch = s.pool_epoch;
    return slot->buffer;
  }
  CqlBuffer* b = cqlcuda_buffer_import_host_readonly(host_ptr, size);
  if (slot)
  {
    cqlcuda_buffer_release(slot->buffer);
    slot->buffer = b;
    slot->capacity = b ? size : 0;
    slot->imported_host_ptr = b ? host_ptr : nullptr;
    slot->last_epoch = s.pool_epoch;
    return b;
  }
  s.pool.push_back(CqlPooled{key, b, b ? size : 0, s.pool_epoch, b ? host_ptr : nullptr});
  s.pool_index[key] = s.pool.size() - 1;
  return b;
}

extern "C" void cqlcuda_buffer_release(CqlBuffer* b)
{
  if (!b) return;
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  // a pooled slot that still points at this buffer forgets it
  for (auto& p : s.pool)
  {
    if (p.buffer == b)
    {
      p.buffer = nullptr;
      p.capacity = 0;
      p.imported_host_ptr = nullptr;
    }
  }
  if (b->imported == 1) cudaHostUnregister(const_cast<void*>(b->host_ptr));
  else if (b->imported == 3) cudaFreeHost(const_cast<void*>(b->host_ptr));
  else if (!b->imported && b->dptr)
  {
    // work already queued on the runtime stream may still read the buffer
    cudaStreamSynchronize(s.stream);
    cudaFree(b->dptr);
    s.mem.bytes_in_use -= std::min(b->charge, s.mem.bytes_in_use);
  }
  delete b;
}

extern "C" void cqlcuda_buffer_write(CqlBuffer* b, const void* data, uint64_t size)
{
  if (!b || !data) return;
  if (size > b->size)
  {
    set_error("cqlcuda_buffer_write: write size exceeds buffer size");
    return;
  }
  if (b->imported)
  {
    set_error("cqlcuda_buffer_write: an imported host buffer is read-only");
    return;
  }
  CqlState& s = S();
  if (note_cuda(cudaMemcpyAsync(b->dptr, data, size, cudaMemcpyHostToDevice, s.stream), "buffer_write"))
    wait_stream(s.stream, "buffer_write");
}

extern "C" void cqlcuda_buffer_read(CqlBuffer* b, void* data, uint64_t size)
{
  if (!b || !data) return;
  if (size > b->size)
  {
    set_error("cqlcuda_buffer_read: read size exceeds buffer size");
    return;
  }
  CqlState& s = S();
  if (!note_cuda(cudaMemcpyAsync(data, b->dptr, size, cudaMemcpyDeviceToHost, s.stream), "buffer_read") ||
      !wait_stream(s.stream, "buffer_read"))
  {
    memset(data, 0, size);
  }
}

extern "C" uint64_t cqlcuda_buffer_size(const CqlBuffer* b) { return b ? b->size : 0; }
extern "C" void* cqlcuda_buffer_device_pointer(const CqlBuffer* b) { return b ? b->dptr : nullptr; }

// ---------------------------------------------------------------------------------------------
// kernels

static const CqlKernelDesc* find_builtin(const std::string& name)
{
  const CqlKernelDesc* tables[] = { cql_kernels_aggregate, cql_kernels_scan, cql_kernels_hash, cql_kernels_join, cql_kernels_sort, cql_kernels_fixed,
                                    cql_kernels_window };
  for (const CqlKernelDesc* t : tables)
  {
    for (const CqlKernelDesc* d = t; d->name; d++)
    {
      if (name == d->name) return d;
    }
  }
  return nullptr;
}

static CqlKernel* kernel_new(const std::string& name)
{
  CqlKernel* k = new CqlKernel();
  k->name = name;
  k->builtin = nullptr;
  k->generated = nullptr;
  k->library = nullptr;
  k->last_use = 0;
  k->gen_block = 256;
  k->gen_smem = 0;
  k->gen_per_sm = 4;
  memset(&k->args, 0, sizeof(k->args));
  memset(k->spec, 0, sizeof(k->spec));
  k->spec_count = 0;
  k->profile_index = profile_slot(name);
  return k;
}

extern "C" CqlKernel* cqlcuda_kernel_alloc(const char* name, uint64_t name_len)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  if (!ensure_init()) return nullptr;
  std::string key(name, name_len);
  auto it = s.kernels.find(key);
  if (it != s.kernels.end())
  {
    if (it->second->generated) it->second->last_use = ++s.kernel_tick;
    return it->second;
  }
  const CqlKernelDesc* d = find_builtin(key);
  if (!d)
  {
    set_error("cqlcuda_kernel_alloc: no kernel named '%s'", key.c_str());
    return nullptr;
  }
  CqlKernel* k = kernel_new(key);
  k->builtin = d->launch;
  s.kernels[key] = k;
  return k;
}

// A generated source may declare its launch shape in a first-line comment:
//   // cql: block=256 smem=0 per_sm=4
static void parse_generated_policy(const std::string& src, CqlKernel* k)
{
  size_t at = src.find("// cql:");
  if (at == std::string::npos) return;
  size_t end = src.find('\n', at);
  std::string line = src.substr(at, end == std::string::npos ? std::string::npos : end - at);
  unsigned v = 0;
  size_t p;
  if ((p = line.find("block=")) != std::string::npos && sscanf(line.c_str() + p, "block=%u", &v) == 1 && v >= 32 && v <= 1024) k->gen_block = v;
  if ((p = line.find("smem=")) != std::string::npos && sscanf(line.c_str() + p, "smem=%u", &v) == 1) k->gen_smem = v;
  if ((p = line.find("per_sm=")) != std::string::npos && sscanf(line.c_str() + p, "per_sm=%u", &v) == 1 && v >= 1 && v <= 32) k->gen_per_sm = v;
}

static uint64_t fnv1a(const void* data, uint64_t n)
{
  const unsigned char* p = (const unsigned char*)data;
  uint64_t h = 1469598103934665603ull;
  for (uint64_t i = 0; i < n; i++)
  {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

static std::vector<char> compile_nvrtc(const std::string& src, const std::string& name, int* ok)
{
  CqlState& s = S();
  std::vector<char> cubin;
  *ok = 0;
  s.compile_attempts += 1;
  if (s.fail_compile_every && (s.compile_attempts % s.fail_compile_every) == 0)
  {
    s.compile_log = "injected compile failure";
    set_error("cqlcuda: injected NVRTC failure for '%s'", name.c_str());
    return cubin;
  }
  // disk cache: key = source hash + a check hash + target + NVRTC version
  int maj = 0, min = 0;
  nvrtcVersion(&maj, &min);
  uint64_t h1 = fnv1a(src.data(), src.size());
  uint64_t h2 = 0;
  for (size_t i = 0; i < src.size(); i++) h2 = h2 * 131 + (unsigned char)src[i];
  char fname[512];
  if (!s.cache_dir.empty())
  {
    snprintf(fname, sizeof(fname), "%s/cql_%016llx%016llx_sm103a_nvrtc%d.%d.cubin", s.cache_dir.c_str(), (unsigned long long)h1,
             (unsigned long long)h2, maj, min);
    FILE* f = fopen(fname, "rb");
    if (f)
    {
      fseek(f, 0, SEEK_END);
      long n = ftell(f);
      fseek(f, 0, SEEK_SET);
      if (n > 0)
      {
        cubin.resize((size_t)n);
        if (fread(cubin.data(), 1, (size_t)n, f) == (size_t)n)
        {
          fclose(f);
          *ok = 1;
          return cubin;
        }
      }
      fclose(f);
      cubin.clear();
    }
  }
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, src.c_str(), (name + ".cu").c_str(), 0, nullptr, nullptr) != NVRTC_SUCCESS)
  {
    set_error("cqlcuda: nvrtcCreateProgram failed for '%s'", name.c_str());
    return cubin;
  }
  const char* opts[] = { "--gpu-architecture=sm_103a", "--std=c++17", "-default-device", "-lineinfo" };
  nvrtcResult r = nvrtcCompileProgram(prog, 4, opts);
  size_t log_size = 0;
  nvrtcGetProgramLogSize(prog, &log_size);
  s.compile_log.assign(log_size, '\0');
  if (log_size) nvrtcGetProgramLog(prog, &s.compile_log[0]);
  if (r != NVRTC_SUCCESS)
  {
    set_error("cqlcuda: NVRTC failed for '%s': %s", name.c_str(), nvrtcGetErrorString(r));
    nvrtcDestroyProgram(&prog);
    return cubin;
  }
  size_t n = 0;
  nvrtcGetCUBINSize(prog, &n);
  cubin.resize(n);
  nvrtcGetCUBIN(prog, cubin.data());
  nvrtcDestroyProgram(&prog);
  s.generated_compiles += 1;
  if (!s.cache_dir.empty())
  {
    FILE* f = fopen(fname, "wb");
    if (f)
    {
      fwrite(cubin.data(), 1, cubin.size(), f);
      fclose(f);
    }
  }
  *ok = 1;
  return cubin;
}

static void graphs_drop_kernel(const CqlKernel* k);

// Evicts the least recently looked-up generated kernels until at most generated_cap stay loaded. Not
// while the main lane's batch is open (its dispatches may name any kernel; the next compile outside a
// batch catches up), and never one of the 8 most recently looked-up. The GPU is drained first, every
// plan graph that launches the kernel is dropped, and its module is unloaded; the kernel object stays
// valid (a stale handle fails its dispatch with an error instead of launching freed code).
static void generated_evict_over_cap(void)
{
  CqlState& s = S();
  // a persistent kernel may run for its idle limit: the device drain below would wait for it
  if (s.main_lane.batch.active || s.persistent_open) return;
  for (;;)
  {
    uint32_t loaded = 0;
    CqlKernel* victim = nullptr;
    for (auto& kv : s.kernels)
    {
      CqlKernel* k = kv.second;
      if (!k->generated) continue;
      loaded += 1;
      if (k->last_use + CQL_GENERATED_KERNEL_MIN_CAP > s.kernel_tick) continue;
      if (!victim || k->last_use < victim->last_use) victim = k;
    }
    if (loaded <= s.generated_cap || !victim) return;
    std::unique_lock<std::shared_mutex> evict(s.generated_use);
    cudaDeviceSynchronize();
    graphs_drop_kernel(victim);
    if (victim->library) cudaLibraryUnload(victim->library);
    cudaGetLastError();
    victim->library = nullptr;
    victim->generated = nullptr;
    s.kernels.erase(victim->name);
    s.retired.push_back(victim);
    s.generated_evictions += 1;
  }
}

extern "C" void cqlcuda_set_generated_kernel_cap(uint32_t cap)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  s.generated_cap = cap < CQL_GENERATED_KERNEL_MIN_CAP ? CQL_GENERATED_KERNEL_MIN_CAP : cap;
  if (s.initialized) generated_evict_over_cap();
}

extern "C" CqlKernel* cqlcuda_kernel_alloc_from_image_spec(const char* name, uint64_t name_len, const void* image, uint64_t image_len,
                                                          const uint32_t* spec_values, uint32_t spec_count)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  if (!ensure_init()) return nullptr;
  std::string key(name, name_len);
  if (spec_count)
  {
    // a specialisation is its own kernel object
    char suffix[32];
    for (uint32_t i = 0; i < spec_count; i++)
    {
      snprintf(suffix, sizeof(suffix), ":%u", spec_values[i]);
      key += suffix;
    }
  }
  auto it = s.kernels.find(key);
  if (it != s.kernels.end())
  {
    if (it->second->generated) it->second->last_use = ++s.kernel_tick;
    return it->second;
  }
  if (!image || image_len == 0)
  {
    return nullptr;  // lookup only (src/gpu/gpu.h:129-130)
  }
  const unsigned char* bytes = (const unsigned char*)image;
  std::vector<char> cubin;
  int is_elf = image_len >= 4 && bytes[0] == 0x7f && bytes[1] == 'E' && bytes[2] == 'L' && bytes[3] == 'F';
  std::string src;
  if (is_elf) cubin.assign((const char*)image, (const char*)image + image_len);
  else
  {
    src.assign((const char*)image, image_len);
    if (spec_count)
    {
      // specialisation constants become preprocessor definitions CQL_SPEC_<i>
      std::string defs;
      char line[64];
      for (uint32_t i = 0; i < spec_count; i++)
      {
        snprintf(line, sizeof(line), "#define CQL_SPEC_%u %uu\n", i, spec_values[i]);
        defs += line;
      }
      src = defs + src;
    }
    int ok = 0;
    cubin = compile_nvrtc(src, key, &ok);
    if (!ok) return nullptr;
  }
  cudaLibrary_t lib = nullptr;
  if (!note_cuda(cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0), "cudaLibraryLoadData")) return nullptr;
  cudaKernel_t kfn = nullptr;
  if (!note_cuda(cudaLibraryGetKernel(&kfn, lib, "cql_main"), "cudaLibraryGetKernel(cql_main)"))
  {
    cudaLibraryUnload(lib);
    return nullptr;
  }
  CqlKernel* k = kernel_new(key);
  k->generated = kfn;
  k->library = lib;
  k->last_use = ++s.kernel_tick;
  if (!src.empty()) parse_generated_policy(src, k);
  if (k->gen_smem > 48 * 1024)
  {
    cudaFuncSetAttribute((const void*)kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k->gen_smem);
  }
  if (spec_count)
  {
    memcpy(k->spec, spec_values, sizeof(uint32_t) * std::min<uint32_t>(spec_count, 16));
    k->spec_count = spec_count;
  }
  s.kernels[key] = k;
  generated_evict_over_cap();
  return k;
}

extern "C" CqlKernel* cqlcuda_kernel_alloc_from_image(const char* name, uint64_t name_len, const void* image, uint64_t image_len)
{
  return cqlcuda_kernel_alloc_from_image_spec(name, name_len, image, image_len, nullptr, 0);
}

extern "C" void cqlcuda_generated_kernel_stats(uint64_t* out_compiles, uint64_t* out_evictions)
{
  if (out_compiles) *out_compiles = S().generated_compiles;
  if (out_evictions) *out_evictions = S().generated_evictions;
}

extern "C" void cqlcuda_kernel_release(CqlKernel*) {}

extern "C" void cqlcuda_kernel_set_arg_buffer(CqlKernel* k, uint32_t index, CqlBuffer* b)
{
  if (!k) return;
  if (index >= CQL_MAX_BINDINGS)
  {
    set_error("cqlcuda_kernel_set_arg_buffer: index %u exceeds %u", index, CQL_MAX_BINDINGS);
    return;
  }
  if (!b)
  {
    set_error("cqlcuda_kernel_set_arg_buffer: buffer argument for index %u is NULL - a prior GPU buffer allocation failed", index);
    return;
  }
  CqlLaunch& A = L().args[k];
  A.buf[index] = b->dptr;
  A.bytes[index] = b->size;
}

extern "C" void cqlcuda_kernel_set_arg_buffer_range(CqlKernel* k, uint32_t index, CqlBuffer* b, uint64_t offset, uint64_t size)
{
  if (!k || !b || index >= CQL_MAX_BINDINGS) return;
  if (offset > b->size || size > b->size - offset)
  {
    set_error("cqlcuda_kernel_set_arg_buffer_range: range [%llu, +%llu) outside a %llu byte buffer", (unsigned long long)offset,
              (unsigned long long)size, (unsigned long long)b->size);
    return;
  }
  CqlLaunch& A = L().args[k];
  A.buf[index] = (char*)b->dptr + offset;
  A.bytes[index] = size;
}

extern "C" void cqlcuda_kernel_set_arg_u64(CqlKernel* k, uint32_t index, uint64_t value)
{
  if (!k) return;
  if (index >= CQL_PUSH_SLOTS)
  {
    set_error("cqlcuda_kernel_set_arg_u64: index %u exceeds %u", index, CQL_PUSH_SLOTS);
    return;
  }
  L().args[k].push[index] = value;
}

// Enqueues one dispatch on `stream`, bracketed by events when the profile is on.
static int dispatch_args(CqlKernel* k, const CqlLaunch& args, uint32_t gws, uint32_t lws, cudaStream_t stream, std::vector<CqlTiming>* timings);

static int dispatch(CqlKernel* k, uint32_t gws, uint32_t lws, cudaStream_t stream, std::vector<CqlTiming>* timings)
{
  return dispatch_args(k, L().args[k], gws, lws, stream, timings);
}

static int dispatch_args(CqlKernel* k, const CqlLaunch& args, uint32_t gws, uint32_t lws, cudaStream_t stream, std::vector<CqlTiming>* timings)
{
  CqlState& s = S();
  if (s.device_lost)
  {
    set_error("cqlcuda: device lost, dispatch of '%s' skipped", k->name.c_str());
    return 0;
  }
  CqlTiming t;
  int timed = s.profile_enabled && timings;
  if (timed)
  {
    t.profile_index = k->profile_index;
    t.start = timing_event_get();
    t.stop = timing_event_get();
    cudaEventRecord(t.start, stream);
  }
  int rc = 0;
  if (!k->builtin && !k->generated)
  {
    set_error("cqlcuda: kernel '%s' was evicted from the generated-kernel cache; look it up again", k->name.c_str());
    return 0;
  }
  if (k->builtin)
  {
    rc = k->builtin(args, gws, lws, stream);
  }
  else
  {
    // a lane launches without the state lock: the eviction of this kernel's module waits for the launch,
    // and a launch after it sees the kernel gone
    std::shared_lock<std::shared_mutex> use(s.generated_use);
    if (!k->generated)
    {
      set_error("cqlcuda: kernel '%s' was evicted from the generated-kernel cache; look it up again", k->name.c_str());
      return 0;
    }
    uint32_t block = k->gen_block;
    uint64_t want = lws ? ((uint64_t)gws + lws - 1) / lws : 1;
    uint32_t grid = cql_stream_grid(want ? want : 1, (int)k->gen_per_sm);
    CqlLaunch a = args;
    void* params[] = { &a };
    cudaError_t e = cudaLaunchKernel((const void*)k->generated, dim3(grid), dim3(block), params, k->gen_smem, stream);
    rc = (int)e;
    if (e == cudaSuccess) cql_note_launch();
  }
  if (timed)
  {
    cudaEventRecord(t.stop, stream);
    timings->push_back(t);
  }
  if (rc != 0)
  {
    note_cuda((cudaError_t)rc, k->name.c_str());
    return 0;
  }
  return 1;
}

extern "C" void cqlcuda_kernel_execute(CqlKernel* k, uint32_t gws, uint32_t lws)
{
  if (!k) return;
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  cudaEventRecord(s.exec_start, s.stream);
  std::vector<CqlTiming> timings;
  int ok = dispatch(k, gws, lws, s.stream, &timings);
  cudaEventRecord(s.exec_stop, s.stream);
  if (ok && wait_stream(s.stream, k->name.c_str()))
  {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, s.exec_start, s.exec_stop) == cudaSuccess) s.last_kernel_us = (uint64_t)(ms * 1000.0f);
    timings_collect(timings);
  }
}

// ---------------------------------------------------------------------------------------------
// pinned staging for reads

static unsigned char* staging_reserve(CqlStaging& st, uint64_t size, uint64_t* out_offset)
{
  uint64_t offset = (st.used + 15) & ~15ull;
  if (offset + size > st.capacity)
  {
    // growing while reads are pending would move them: callers size the staging at begin
    if (!st.reads.empty()) return nullptr;
    uint64_t cap = std::max<uint64_t>(offset + size, std::max<uint64_t>(st.capacity * 2, 1 << 16));
    unsigned char* p = nullptr;
    if (cudaHostAlloc((void**)&p, cap, cudaHostAllocDefault) != cudaSuccess)
    {
      cudaGetLastError();
      return nullptr;
    }
    if (st.host) cudaFreeHost(st.host);
    st.host = p;
    st.capacity = cap;
  }
  st.used = offset + size;
  *out_offset = offset;
  return st.host + offset;
}

static void staging_prepare(CqlStaging& st, uint64_t bytes)
{
  st.used = 0;
  st.reads.clear();
  if (bytes + 4096 > st.capacity)
  {
    uint64_t unused;
    staging_reserve(st, bytes + 4096, &unused);
    st.used = 0;
  }
}

static void staging_finish(CqlStaging& st, int ok)
{
  for (auto& r : st.reads)
  {
    if (ok) memcpy(r.dst, st.host + r.staging_offset, r.size);
    else memset(r.dst, 0, r.size);
  }
  st.reads.clear();
  st.used = 0;
}

// Reads from this size on go straight to the caller's memory. On GB300 a device-to-host copy into pageable
// memory runs at 64 GB/s for 1 MB and 154 GB/s for 8 MB (measured), while a read through the staging area
// also pays a host memcpy of about 14 GB/s.
#define CQL_DIRECT_READ_BYTES (256ull << 10)

static int enqueue_read(CqlStaging& st, CqlBuffer* b, uint64_t offset, void* out, uint64_t size, cudaStream_t stream, bool allow_direct = true)
{
  if (!b || !out) return 0;
  if (offset > b->size || size > b->size - offset)
  {
    set_error("cqlcuda: read of %llu bytes at %llu from a %llu byte buffer", (unsigned long long)size, (unsigned long long)offset,
              (unsigned long long)b->size);
    return 0;
  }
  const char* src = (const char*)b->dptr + offset;
  uint64_t off = 0;
  // a large result goes straight to the caller's memory (the copy waits for the work before it):
  // through a staging area it would cross host memory twice
  unsigned char* dst = (allow_direct && size >= CQL_DIRECT_READ_BYTES) ? nullptr : staging_reserve(st, size, &off);
  if (!dst)
  {
    if (!note_cuda(cudaMemcpyAsync(out, src, size, cudaMemcpyDeviceToHost, stream), "read")) return 0;
    return wait_stream(stream, "read");
  }
  if (!note_cuda(cudaMemcpyAsync(dst, src, size, cudaMemcpyDeviceToHost, stream), "read")) return 0;
  st.reads.push_back(CqlPendingRead{out, off, size});
  return 1;
}

// ---------------------------------------------------------------------------------------------
// batches: one active at a time (src/gpu/vulkan/gpu_vulkan.h:215)

extern "C" CqlBatch* cqlcuda_batch_begin(uint64_t upload_bytes_needed, uint64_t download_bytes_needed)
{
  CqlState& s = S();
  CqlLane& l = L();
  // the main lane holds one batch at a time (src/gpu/vulkan/gpu_vulkan.h:215); a thread's own lane needs no lock
  if (l.is_main) s.lock.lock();
  if (!ensure_init())
  {
    if (l.is_main) s.lock.unlock();
    return nullptr;
  }
  (void)upload_bytes_needed;
  CqlBatch* b = &l.batch;
  b->active = 1;
  b->failed = 0;
  if (s.profile_enabled) b->opened = std::chrono::steady_clock::now();
  b->recording = 0;
  b->ops.clear();
  b->in_bytes.clear();
  b->out_bytes = 0;
  staging_prepare(b->staging, download_bytes_needed);
  return b;
}

extern "C" CqlBatch* cqlcuda_batch_begin_graph(uint64_t upload_bytes_needed, uint64_t download_bytes_needed, uint64_t plan_key)
{
  CqlBatch* b = cqlcuda_batch_begin(upload_bytes_needed, download_bytes_needed);
  // plan graphs are kept to the main lane: a thread's own lane (a serving worker) runs ordinary batches
  if (b && L().is_main)
  {
    b->recording = 1;
    b->plan_key = plan_key;
  }
  return b;
}

static CqlOp op_of(int kind, CqlBuffer* buffer, uint64_t offset, uint64_t size)
{
  CqlOp o;
  memset(&o, 0, sizeof(o));
  o.kind = kind;
  o.buffer = buffer;
  o.dptr = buffer ? buffer->dptr : nullptr;
  o.offset = offset;
  o.size = size;
  return o;
}

extern "C" void cqlcuda_batch_buffer_write(CqlBatch* batch, CqlBuffer* buffer, const void* data, uint64_t size)
{
  if (!batch || !buffer || !data) return;
  if (size > buffer->size || buffer->imported)
  {
    set_error("cqlcuda_batch_buffer_write: bad destination");
    batch->failed = 1;
    return;
  }
  if (batch->recording)
  {
    CqlOp o = op_of(CQL_OP_WRITE, buffer, 0, size);
    o.at = (batch->in_bytes.size() + 15) & ~15ull;
    batch->in_bytes.resize(o.at + size);
    memcpy(batch->in_bytes.data() + o.at, data, size);
    batch->ops.push_back(o);
    return;
  }
  if (!note_cuda(cudaMemcpyAsync(buffer->dptr, data, size, cudaMemcpyHostToDevice, L().stream), "batch write")) batch->failed = 1;
}

extern "C" void cqlcuda_batch_buffer_zero(CqlBatch* batch, CqlBuffer* buffer, uint64_t size)
{
  if (!batch || !buffer) return;
  if (batch->recording)
  {
    batch->ops.push_back(op_of(CQL_OP_ZERO, buffer, 0, std::min(size, buffer->size)));
    return;
  }
  if (!note_cuda(cudaMemsetAsync(buffer->dptr, 0, std::min(size, buffer->size), L().stream), "batch zero")) batch->failed = 1;
}

__global__ void k_fill_u32(uint32_t* p, uint64_t words, uint32_t value)
{
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (; i < words; i += stride) p[i] = value;
}

static int fill_words(CqlBuffer* buffer, uint64_t offset, uint64_t size, uint32_t value, cudaStream_t stream)
{
  if (offset > buffer->size || (offset & 3)) return 0;
  uint64_t bytes = std::min(size, buffer->size - offset);
  char* at = (char*)buffer->dptr + offset;
  if (value == 0 || value == 0xffffffffu || ((value & 0xff) * 0x01010101u) == value)
  {
    return note_cuda(cudaMemsetAsync(at, (int)(value & 0xff), bytes, stream), "fill");
  }
  uint64_t words = bytes / 4;
  if (words == 0) return 1;
  uint32_t grid = cql_stream_grid((words + 255) / 256, 8);
  k_fill_u32<<<grid, 256, 0, stream>>>((uint32_t*)at, words, value);
  cql_note_launch();
  return note_cuda(cudaGetLastError(), "fill");
}

extern "C" void cqlcuda_batch_buffer_fill(CqlBatch* batch, CqlBuffer* buffer, uint64_t size, uint32_t value)
{
  if (!batch || !buffer) return;
  if (batch->recording)
  {
    CqlOp o = op_of(CQL_OP_FILL, buffer, 0, size);
    o.value = value;
    batch->ops.push_back(o);
    return;
  }
  if (!fill_words(buffer, 0, size, value, L().stream)) batch->failed = 1;
}

extern "C" void cqlcuda_batch_fill_range(CqlBatch* batch, CqlBuffer* buffer, uint64_t offset, uint64_t size, uint32_t value)
{
  if (!batch || !buffer) return;
  if (batch->recording)
  {
    CqlOp o = op_of(CQL_OP_FILL, buffer, offset, size);
    o.value = value;
    batch->ops.push_back(o);
    return;
  }
  if (!fill_words(buffer, offset, size, value, L().stream))
  {
    set_error("cqlcuda_batch_fill_range: offset %llu of a %llu byte buffer", (unsigned long long)offset, (unsigned long long)buffer->size);
    batch->failed = 1;
  }
}

extern "C" void cqlcuda_batch_kernel_execute(CqlBatch* batch, CqlKernel* kernel, uint32_t gws, uint32_t lws)
{
  if (!batch || !kernel) return;
  if (batch->recording)
  {
    CqlOp o = op_of(CQL_OP_KERNEL, nullptr, 0, 0);
    o.kernel = kernel;
    o.launch = L().args[kernel];
    o.gws = gws;
    o.lws = lws;
    batch->ops.push_back(o);
    return;
  }
  if (!dispatch(kernel, gws, lws, L().stream, &L().timings)) batch->failed = 1;
}

extern "C" void cqlcuda_batch_buffer_read(CqlBatch* batch, CqlBuffer* buffer, void* out_data, uint64_t size)
{
  if (!batch) return;
  if (!buffer)
  {
    if (out_data) memset(out_data, 0, size);
    return;
  }
  cqlcuda_batch_buffer_read_at(batch, buffer, 0, out_data, size);
}

extern "C" void cqlcuda_batch_buffer_read_at(CqlBatch* batch, CqlBuffer* buffer, uint64_t offset, void* out_data, uint64_t size)
{
  if (!batch) return;
  if (!buffer)
  {
    if (out_data) memset(out_data, 0, size);
    return;
  }
  if (batch->recording)
  {
    if (!out_data || offset > buffer->size || size > buffer->size - offset)
    {
      set_error("cqlcuda: read of %llu bytes at %llu from a %llu byte buffer", (unsigned long long)size, (unsigned long long)offset,
                (unsigned long long)buffer->size);
      batch->failed = 1;
      return;
    }
    CqlOp o = op_of(CQL_OP_READ, buffer, offset, size);
    o.out = out_data;
    o.at = (batch->out_bytes + 15) & ~15ull;
    batch->out_bytes = o.at + size;
    batch->ops.push_back(o);
    return;
  }
  if (!enqueue_read(batch->staging, buffer, offset, out_data, size, L().stream)) batch->failed = 1;
}

// ---------------------------------------------------------------------------------------------
// plan graphs

#define CQL_GRAPHS_PER_LANE 32

static uint64_t fnv_bytes(uint64_t h, const void* p, size_t n)
{
  const unsigned char* c = (const unsigned char*)p;
  for (size_t i = 0; i < n; i++) h = (h ^ c[i]) * 1099511628211ull;
  return h;
}

// what a replay must match: every operation with its buffer addresses, sizes, fill values and kernel
// arguments, and where its bytes sit in the record (the bytes themselves are the replay's new input)
static uint64_t record_fingerprint(const CqlBatch* b)
{
  uint64_t h = fnv_bytes(1469598103934665603ull, &b->plan_key, 8);
  h = fnv_bytes(h, &b->out_bytes, 8);
  uint64_t in = b->in_bytes.size();
  h = fnv_bytes(h, &in, 8);
  for (const CqlOp& o : b->ops)
  {
    h = fnv_bytes(h, &o.kind, sizeof(o.kind));
    h = fnv_bytes(h, &o.dptr, sizeof(o.dptr));
    h = fnv_bytes(h, &o.offset, 8);
    h = fnv_bytes(h, &o.size, 8);
    h = fnv_bytes(h, &o.value, 4);
    h = fnv_bytes(h, &o.at, 8);
    if (o.kind == CQL_OP_KERNEL)
    {
      h = fnv_bytes(h, &o.kernel, sizeof(o.kernel));
      h = fnv_bytes(h, &o.launch, sizeof(o.launch));
      h = fnv_bytes(h, &o.gws, 4);
      h = fnv_bytes(h, &o.lws, 4);
    }
  }
  return h;
}

// the record's operations on the stream; `in`/`out` are the graph's pinned areas, or null for an eager
// run (bytes from the record, results through the batch's staging)
static int issue_ops(CqlBatch* b, cudaStream_t stream, const unsigned char* in, unsigned char* out, uint32_t* kernels)
{
  for (const CqlOp& o : b->ops)
  {
    int ok = 1;
    switch (o.kind)
    {
      case CQL_OP_WRITE:
        ok = note_cuda(cudaMemcpyAsync(o.buffer->dptr, (in ? in : b->in_bytes.data()) + o.at, o.size, cudaMemcpyHostToDevice, stream), "graph write");
        break;
      case CQL_OP_ZERO: ok = note_cuda(cudaMemsetAsync(o.buffer->dptr, 0, o.size, stream), "graph zero"); break;
      case CQL_OP_FILL: ok = fill_words(o.buffer, o.offset, o.size, o.value, stream); break;
      case CQL_OP_KERNEL:
        ok = dispatch_args(o.kernel, o.launch, o.gws, o.lws, stream, out ? nullptr : &L().timings);
        if (kernels) *kernels += 1;
        break;
      default:
        if (out) ok = note_cuda(cudaMemcpyAsync(out + o.at, (const char*)o.buffer->dptr + o.offset, o.size, cudaMemcpyDeviceToHost, stream), "graph read");
        else ok = enqueue_read(b->staging, o.buffer, o.offset, o.out, o.size, stream);
        break;
    }
    if (!ok) return 0;
  }
  return 1;
}

static void graph_entry_free(CqlGraphEntry& e)
{
  if (e.exec) cudaGraphExecDestroy(e.exec);
  if (e.in) cudaFreeHost(e.in);
  if (e.out) cudaFreeHost(e.out);
  e.exec = nullptr;
  e.in = e.out = nullptr;
  e.ops.clear();
}

// a fingerprint hit replays only when the record is the captured one, field by field (everything the
// fingerprint covers; the callers' destinations and the bytes written may differ)
static bool record_equals(const CqlBatch* b, const CqlGraphEntry& e)
{
  if (b->plan_key != e.plan_key || b->out_bytes != e.out_size || b->in_bytes.size() != e.in_size || b->ops.size() != e.ops.size()) return false;
  for (size_t i = 0; i < b->ops.size(); i++)
  {
    const CqlOp& x = b->ops[i];
    const CqlOp& y = e.ops[i];
    if (x.kind != y.kind || x.dptr != y.dptr || x.offset != y.offset || x.size != y.size || x.value != y.value || x.at != y.at) return false;
    if (x.kind == CQL_OP_KERNEL &&
        (x.kernel != y.kernel || x.gws != y.gws || x.lws != y.lws || memcmp(&x.launch, &y.launch, sizeof(CqlLaunch)) != 0))
      return false;
  }
  return true;
}

// plan graphs that launch an evicted kernel go with it (graphs live on the main lane only)
static void graphs_drop_kernel(const CqlKernel* k)
{
  CqlLane& l = S().main_lane;
  for (auto it = l.graphs.begin(); it != l.graphs.end();)
  {
    bool uses = false;
    for (const CqlOp& o : it->second.ops)
      if (o.kind == CQL_OP_KERNEL && o.kernel == k) uses = true;
    if (uses)
    {
      graph_entry_free(it->second);
      it = l.graphs.erase(it);
    }
    else ++it;
  }
}

static void graph_copy_out(CqlBatch* b, const CqlGraphEntry& e)
{
  for (const CqlOp& o : b->ops)
    if (o.kind == CQL_OP_READ) memcpy(o.out, e.out + o.at, o.size);
}

// Replays the graph of the record's shape, or captures one; falls back to issuing the record eagerly
// when a capture does not take. The results reach the callers' arrays before it returns.
static void graph_end(CqlBatch* b, CqlLane& l)
{
  if (S().profile_enabled || !g_graphs_on.load())
  {
    // a profiled batch times every kernel with events of its own: it runs eagerly
    if (!issue_ops(b, l.stream, nullptr, nullptr, nullptr)) b->failed = 1;
    b->recording = 0;
    return;
  }
  uint64_t fp = record_fingerprint(b);
  auto it = l.graphs.find(fp);
  if (it != l.graphs.end() && !record_equals(b, it->second))
  {
    // two shapes with one fingerprint: the newcomer runs eagerly, the captured graph stays
    if (!issue_ops(b, l.stream, nullptr, nullptr, nullptr)) b->failed = 1;
    b->recording = 0;
    return;
  }
  if (it != l.graphs.end())
  {
    CqlGraphEntry& e = it->second;
    if (!b->in_bytes.empty()) memcpy(e.in, b->in_bytes.data(), b->in_bytes.size());
    if (!note_cuda(cudaGraphLaunch(e.exec, l.stream), "cudaGraphLaunch") || !wait_stream(l.stream, "graph replay"))
    {
      b->failed = 1;
      return;
    }
    for (uint32_t i = 0; i < e.kernels; i++) cql_note_launch();
    e.last_use = ++l.graph_clock;
    g_graph_replays.fetch_add(1, std::memory_order_relaxed);
    graph_copy_out(b, e);
    return;
  }
  // a shape is captured the second time it is met: a capture and its instantiation cost more than the
  // launches a graph saves, so shapes met once (a serving loop's odd batch sizes) run eagerly
  if (l.graph_seen.find(fp) == l.graph_seen.end())
  {
    if (l.graph_seen.size() >= 4096) l.graph_seen.clear();
    l.graph_seen[fp] = 1;
    if (!issue_ops(b, l.stream, nullptr, nullptr, nullptr)) b->failed = 1;
    b->recording = 0;
    return;
  }
  CqlGraphEntry e{};
  e.in_size = b->in_bytes.size();
  e.out_size = b->out_bytes;
  e.plan_key = b->plan_key;
  e.ops = b->ops;
  bool pinned = cudaHostAlloc((void**)&e.in, std::max<uint64_t>(e.in_size, 16), cudaHostAllocDefault) == cudaSuccess &&
                cudaHostAlloc((void**)&e.out, std::max<uint64_t>(e.out_size, 16), cudaHostAllocDefault) == cudaSuccess;
  cudaGraph_t graph = nullptr;
  bool captured = false;
  if (pinned)
  {
    if (e.in_size) memcpy(e.in, b->in_bytes.data(), e.in_size);
    if (cudaStreamBeginCapture(l.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess)
    {
      bool issued = issue_ops(b, l.stream, e.in, e.out, &e.kernels) != 0;
      cudaError_t end = cudaStreamEndCapture(l.stream, &graph);
      captured = issued && end == cudaSuccess && graph &&
                 cudaGraphInstantiate(&e.exec, graph, 0) == cudaSuccess;
      if (graph) cudaGraphDestroy(graph);
    }
  }
  cudaGetLastError();
  if (!captured)
  {
    // the record runs as an ordinary batch
    graph_entry_free(e);
    g_graph_fallbacks.fetch_add(1, std::memory_order_relaxed);
    set_error("");
    if (!issue_ops(b, l.stream, nullptr, nullptr, nullptr)) b->failed = 1;
    // eager reads wait in the batch's staging: hand the record's reads over to it
    b->recording = 0;
    return;
  }
  if (!note_cuda(cudaGraphLaunch(e.exec, l.stream), "cudaGraphLaunch") || !wait_stream(l.stream, "graph launch"))
  {
    graph_entry_free(e);
    b->failed = 1;
    return;
  }
  g_graph_captures.fetch_add(1, std::memory_order_relaxed);
  graph_copy_out(b, e);
  if (l.graphs.size() >= CQL_GRAPHS_PER_LANE)
  {
    auto oldest = l.graphs.begin();
    for (auto j = l.graphs.begin(); j != l.graphs.end(); ++j)
      if (j->second.last_use < oldest->second.last_use) oldest = j;
    graph_entry_free(oldest->second);
    l.graphs.erase(oldest);
  }
  e.last_use = ++l.graph_clock;
  l.graphs[fp] = e;
}

extern "C" void cqlcuda_graph_enable(int on) { g_graphs_on.store(on ? 1 : 0); }

extern "C" void cqlcuda_graph_stats(uint64_t* out_captures, uint64_t* out_replays, uint64_t* out_fallbacks)
{
  if (out_captures) *out_captures = g_graph_captures.load();
  if (out_replays) *out_replays = g_graph_replays.load();
  if (out_fallbacks) *out_fallbacks = g_graph_fallbacks.load();
}

extern "C" int cqlcuda_batch_end(CqlBatch* batch)
{
  CqlState& s = S();
  if (!batch)
  {
    return 0;
  }
  CqlLane& l = L();
  const bool host_timed = s.profile_enabled != 0;
  auto t_end = host_timed ? std::chrono::steady_clock::now() : std::chrono::steady_clock::time_point();
  if (batch->recording && !batch->failed) graph_end(batch, l);
  int ok = !batch->failed && wait_stream(l.stream, "batch_end");
  auto t_waited = host_timed ? std::chrono::steady_clock::now() : t_end;
  if (batch->recording)
  {
    // the results of a recorded batch were copied from its graph's out area (or its staging, eagerly)
    for (const CqlOp& o : batch->ops)
      if (o.kind == CQL_OP_READ && !ok) memset(o.out, 0, o.size);
    batch->recording = 0;
  }
  staging_finish(batch->staging, ok);
  if (host_timed)
  {
    // host-side totals beside the kernels' (cqlcuda_host_profile): a batch from its opening to its end, the
    // wait for its work, and the copies of staged results into the callers' arrays
    auto t_done = std::chrono::steady_clock::now();
    auto ns = [](std::chrono::steady_clock::duration d) { return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(d).count(); };
    s.host_open_ns.fetch_add(ns(t_done - batch->opened));
    s.host_wait_ns.fetch_add(ns(t_waited - t_end));
    s.host_copy_ns.fetch_add(ns(t_done - t_waited));
    s.host_batches.fetch_add(1);
  }
  if (ok) timings_collect(l.timings);
  else
  {
    for (auto& t : l.timings)
    {
      timing_event_put(t.start);
      timing_event_put(t.stop);
    }
    l.timings.clear();
  }
  batch->active = 0;
  if (l.is_main) s.lock.unlock();
  return ok;
}

// ---------------------------------------------------------------------------------------------
// streams

extern "C" CqlStream* cqlcuda_stream_alloc(uint32_t slot_count)
{
  if (!ensure_init()) return nullptr;
  if (slot_count == 0 || slot_count > 8)
  {
    set_error("cqlcuda_stream_alloc: %u slots, 1 to 8 allowed", slot_count);
    return nullptr;
  }
  CqlStream* st = new CqlStream();
  st->slot_count = slot_count;
  memset(&st->stats, 0, sizeof(st->stats));
  st->stats.separate_copy_queue = 1;
  for (uint32_t i = 0; i < slot_count; i++)
  {
    CqlStreamSlot& sl = st->slots[i];
    if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess)
    {
      set_error("cqlcuda_stream_alloc: stream creation failed");
      for (uint32_t j = 0; j < i; j++)
      {
        cudaStreamDestroy(st->slots[j].stream);
        cudaEventDestroy(st->slots[j].done);
      }
      delete st;
      return nullptr;
    }
    sl.submitted = 0;
    sl.failed = 0;
    sl.staging.host = nullptr;
    sl.staging.capacity = 0;
    sl.staging.used = 0;
  }
  // slots run after everything already queued on the runtime stream
  cudaEvent_t ev;
  cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  cudaEventRecord(ev, S().stream);
  for (uint32_t i = 0; i < slot_count; i++) cudaStreamWaitEvent(st->slots[i].stream, ev, 0);
  cudaEventDestroy(ev);
  return st;
}

extern "C" void cqlcuda_stream_release(CqlStream* st)
{
  if (!st) return;
  for (uint32_t i = 0; i < st->slot_count; i++)
  {
    CqlStreamSlot& sl = st->slots[i];
    wait_stream(sl.stream, "stream_release");
    for (auto& t : sl.timings)
    {
      timing_event_put(t.start);
      timing_event_put(t.stop);
    }
    cudaStreamDestroy(sl.stream);
    cudaEventDestroy(sl.done);
    staging_release(sl.staging);
  }
  delete st;
}

extern "C" int cqlcuda_stream_slot_begin(CqlStream* st, uint32_t slot, uint64_t upload_bytes, uint64_t readback_bytes)
{
  if (!st || slot >= st->slot_count) return 0;
  CqlStreamSlot& sl = st->slots[slot];
  (void)upload_bytes;
  if (!sl.staging.reads.empty())
  {
    // the previous use of the slot was never waited for
    if (!wait_stream(sl.stream, "stream_slot_begin")) return 0;
    staging_finish(sl.staging, 1);
  }
  sl.submitted = 0;
  sl.failed = 0;
  staging_prepare(sl.staging, readback_bytes);
  return 1;
}

extern "C" int cqlcuda_stream_copy(CqlStream* st, uint32_t slot, CqlBuffer* dst, const void* host_ptr, uint64_t size)
{
  if (!st || slot >= st->slot_count || !dst || !host_ptr) return 0;
  if (size > dst->size || dst->imported)
  {
    set_error("cqlcuda_stream_copy: bad destination");
    return 0;
  }
  CqlStreamSlot& sl = st->slots[slot];
  if (!note_cuda(cudaMemcpyAsync(dst->dptr, host_ptr, size, cudaMemcpyHostToDevice, sl.stream), "stream_copy"))
  {
    sl.failed = 1;
    return 0;
  }
  st->stats.bytes_copied += size;
  return 1;
}

extern "C" void cqlcuda_stream_zero(CqlStream* st, uint32_t slot, CqlBuffer* b, uint64_t size)
{
  if (!st || slot >= st->slot_count || !b) return;
  if (!note_cuda(cudaMemsetAsync(b->dptr, 0, std::min(size, b->size), st->slots[slot].stream), "stream_zero")) st->slots[slot].failed = 1;
}

extern "C" void cqlcuda_stream_fill(CqlStream* st, uint32_t slot, CqlBuffer* b, uint64_t size, uint32_t value)
{
  if (!st || slot >= st->slot_count || !b) return;
  if (!fill_words(b, 0, size, value, st->slots[slot].stream)) st->slots[slot].failed = 1;
}

extern "C" void cqlcuda_stream_dispatch(CqlStream* st, uint32_t slot, CqlKernel* k, uint32_t gws, uint32_t lws)
{
  if (!st || slot >= st->slot_count || !k) return;
  if (!dispatch(k, gws, lws, st->slots[slot].stream, &st->slots[slot].timings)) st->slots[slot].failed = 1;
}

extern "C" void cqlcuda_stream_read(CqlStream* st, uint32_t slot, CqlBuffer* b, void* out, uint64_t size)
{
  if (!st || slot >= st->slot_count) return;
  if (!enqueue_read(st->slots[slot].staging, b, 0, out, size, st->slots[slot].stream, false)) st->slots[slot].failed = 1;
}

extern "C" int cqlcuda_stream_submit(CqlStream* st, uint32_t slot)
{
  if (!st || slot >= st->slot_count) return 0;
  CqlStreamSlot& sl = st->slots[slot];
  if (!note_cuda(cudaEventRecord(sl.done, sl.stream), "stream_submit")) return 0;
  sl.submitted = 1;
  return !sl.failed;
}

extern "C" int cqlcuda_stream_wait(CqlStream* st, uint32_t slot)
{
  if (!st || slot >= st->slot_count) return 0;
  CqlStreamSlot& sl = st->slots[slot];
  int ok = !sl.failed;
  if (sl.submitted) ok = wait_event(sl.done, "stream_wait") && ok;
  else ok = wait_stream(sl.stream, "stream_wait") && ok;
  staging_finish(sl.staging, ok);
  if (ok) timings_collect(sl.timings);
  sl.submitted = 0;
  return ok;
}

extern "C" CqlStreamStats cqlcuda_stream_get_stats(CqlStream* st)
{
  CqlStreamStats z;
  memset(&z, 0, sizeof(z));
  return st ? st->stats : z;
}

// ---------------------------------------------------------------------------------------------
// hooks and diagnostics

extern "C" void cqlcuda_set_fault_alloc_at(uint64_t call_index) { S().fault_alloc_at = call_index; }
extern "C" void cqlcuda_set_evict_hook(CqlEvictHook hook) { S().evict_hook = hook; }
extern "C" void cqlcuda_kernel_profile_enable(int enabled) { S().profile_enabled = enabled; }

// while the kernel profile is on: batches ended, and their host-side time (opening to end, waiting for the
// device, copying staged results), since the last profile reset
extern "C" void cqlcuda_host_profile(uint64_t* out_batches, uint64_t* out_open_ns, uint64_t* out_wait_ns, uint64_t* out_copy_ns)
{
  CqlState& s = S();
  if (out_batches) *out_batches = s.host_batches.load();
  if (out_open_ns) *out_open_ns = s.host_open_ns.load();
  if (out_wait_ns) *out_wait_ns = s.host_wait_ns.load();
  if (out_copy_ns) *out_copy_ns = s.host_copy_ns.load();
}
extern "C" void cqlcuda_kernel_profile_reset(void)
{
  CqlState& s = S();
  for (auto& p : s.profile)
  {
    p.total_ns = 0;
    p.dispatches = 0;
  }
  s.host_batches = 0;
  s.host_open_ns = 0;
  s.host_wait_ns = 0;
  s.host_copy_ns = 0;
}
extern "C" int cqlcuda_kernel_profile_entry(uint32_t index, const char** out_name, uint64_t* out_total_ns, uint64_t* out_dispatches)
{
  CqlState& s = S();
  if (index >= s.profile.size()) return 0;
  if (out_name) *out_name = s.profile[index].name.c_str();
  if (out_total_ns) *out_total_ns = s.profile[index].total_ns;
  if (out_dispatches) *out_dispatches = s.profile[index].dispatches;
  return 1;
}
// a thread with its own lane counts its own launches; otherwise the process's
extern "C" uint32_t cqlcuda_kernel_launch_count(void) { return tl_lane ? tl_lane->launches : S().launches.load(); }
extern "C" const char* cqlcuda_last_error(void) { return tl_error.c_str(); }
extern "C" void cqlcuda_clear_error(void) { tl_error.clear(); }
extern "C" void cqlcuda_set_wait_timeout_ms(uint32_t ms) { S().wait_timeout_ms = ms ? ms : 1; }
extern "C" void cqlcuda_set_module_cache_dir(const char* path) { S().cache_dir = path ? path : ""; }
extern "C" void cqlcuda_set_fail_compile_every(uint32_t n) { S().fail_compile_every = n; }
extern "C" const char* cqlcuda_last_compile_log(void) { return S().compile_log.c_str(); }

extern "C" int cqlcuda_compile_check(const char* source, uint64_t source_len)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  std::string src(source, source_len);
  std::string saved = s.cache_dir;
  s.cache_dir.clear();
  uint32_t fail_every = s.fail_compile_every;
  s.fail_compile_every = 0;
  int ok = 0;
  compile_nvrtc(src, "compile_check", &ok);
  s.cache_dir = saved;
  s.fail_compile_every = fail_every;
  return ok;
}

// ---------------------------------------------------------------------------------------------
// data generation and timing helpers

// splitmix64 (src/tests/bench_common.h:30-37): draw k (0-based) of the stream seeded `seed` is
// mix(seed + (k + 1) * golden), so any draw can be computed on its own.
__device__ __forceinline__ uint64_t splitmix_draw(uint64_t seed, uint64_t k)
{
  uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void k_fill_splitmix(uint32_t* out, uint64_t rows, uint64_t seed, uint32_t per_row, uint32_t index, uint64_t range)
{
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (; i < rows; i += stride)
  {
    uint64_t v = splitmix_draw(seed, i * per_row + index);
    out[i] = (uint32_t)(range ? v % range : v);
  }
}

__global__ void k_fill_sequence(uint32_t* out, uint64_t rows, uint32_t first)
{
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (; i < rows; i += stride) out[i] = first + (uint32_t)i;
}

__global__ void k_fill_affine(uint32_t* out, uint64_t rows, uint64_t mul, uint64_t add, uint64_t modulus)
{
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (; i < rows; i += stride)
  {
    uint64_t v = i * mul + add;
    out[i] = (uint32_t)(modulus ? v % modulus : v);
  }
}

extern "C" int cqlcuda_fill_splitmix_u32(CqlBuffer* b, uint64_t rows, uint64_t seed, uint32_t per_row, uint32_t index, uint64_t range)
{
  if (!b || rows * 4 > b->size || b->imported) return 0;
  CqlState& s = S();
  uint32_t grid = cql_stream_grid((rows + 255) / 256, 8);
  k_fill_splitmix<<<grid, 256, 0, s.stream>>>((uint32_t*)b->dptr, rows, seed, per_row, index, range);
  if (!note_cuda(cudaGetLastError(), "fill_splitmix")) return 0;
  return wait_stream(s.stream, "fill_splitmix");
}

extern "C" int cqlcuda_fill_sequence_u32(CqlBuffer* b, uint64_t rows, uint32_t first)
{
  if (!b || rows * 4 > b->size || b->imported) return 0;
  CqlState& s = S();
  uint32_t grid = cql_stream_grid((rows + 255) / 256, 8);
  k_fill_sequence<<<grid, 256, 0, s.stream>>>((uint32_t*)b->dptr, rows, first);
  if (!note_cuda(cudaGetLastError(), "fill_sequence")) return 0;
  return wait_stream(s.stream, "fill_sequence");
}

extern "C" int cqlcuda_fill_affine_u32(CqlBuffer* b, uint64_t rows, uint64_t mul, uint64_t add, uint64_t modulus)
{
  if (!b || rows * 4 > b->size || b->imported) return 0;
  CqlState& s = S();
  uint32_t grid = cql_stream_grid((rows + 255) / 256, 8);
  k_fill_affine<<<grid, 256, 0, s.stream>>>((uint32_t*)b->dptr, rows, mul, add, modulus);
  if (!note_cuda(cudaGetLastError(), "fill_affine")) return 0;
  return wait_stream(s.stream, "fill_affine");
}

// ---------------------------------------------------------------------------------------------
// page-locked host memory for uploads

static std::mutex g_host_lock;
static std::unordered_map<void*, uint64_t> g_host_blocks;

extern "C" void* cqlcuda_host_alloc(uint64_t bytes)
{
  if (!ensure_init() || bytes == 0) return nullptr;
  long page = sysconf(_SC_PAGESIZE);
  uint64_t size = (bytes + (uint64_t)page - 1) / (uint64_t)page * (uint64_t)page;
  void* p = mmap(nullptr, size, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (p == MAP_FAILED)
  {
    set_error("cqlcuda_host_alloc: mmap of %llu bytes failed", (unsigned long long)size);
    return nullptr;
  }
  // large pages where the kernel offers them, and the pages on the host node nearest the GPU
  madvise(p, size, MADV_HUGEPAGE);
  int node = -1;
  cudaDeviceGetAttribute(&node, cudaDevAttrHostNumaId, S().device);
  if (node >= 0 && node < 1024)
  {
    unsigned long mask[1024 / (8 * sizeof(unsigned long))];
    memset(mask, 0, sizeof(mask));
    mask[node / (8 * sizeof(unsigned long))] |= 1ul << (node % (8 * sizeof(unsigned long)));
    syscall(SYS_mbind, p, size, 1 /* MPOL_PREFERRED */, mask, 1024ul, 0u);
  }
  // every page is written before it is registered: an untouched anonymous page is the shared zero page,
  // and the pinned mapping must be of the page the process will write
  memset(p, 0, size);
  cudaError_t e = cudaHostRegister(p, size, cudaHostRegisterDefault);
  if (e != cudaSuccess)
  {
    cudaGetLastError();
    munmap(p, size);
    set_error("cqlcuda_host_alloc: cudaHostRegister of %llu bytes failed: %s", (unsigned long long)size, cudaGetErrorString(e));
    return nullptr;
  }
  std::lock_guard<std::mutex> g(g_host_lock);
  g_host_blocks[p] = size;
  return p;
}

extern "C" void cqlcuda_host_free(void* p)
{
  if (!p) return;
  uint64_t size = 0;
  {
    std::lock_guard<std::mutex> g(g_host_lock);
    auto it = g_host_blocks.find(p);
    if (it == g_host_blocks.end()) return;
    size = it->second;
    g_host_blocks.erase(it);
  }
  cudaHostUnregister(p);
  munmap(p, size);
}

extern "C" int cqlcuda_flush_l2(uint64_t bytes)
{
  CqlState& s = S();
  if (!ensure_init()) return 0;
  if (s.flush_bytes < bytes)
  {
    if (s.flush_buf) cudaFree(s.flush_buf);
    s.flush_buf = nullptr;
    s.flush_bytes = 0;
    if (cudaMalloc(&s.flush_buf, bytes) != cudaSuccess)
    {
      cudaGetLastError();
      return 0;
    }
    s.flush_bytes = bytes;
  }
  return note_cuda(cudaMemsetAsync(s.flush_buf, 0x5a, bytes, s.stream), "flush_l2");
}

extern "C" void cqlcuda_timer_begin(void)
{
  if (!ensure_init()) return;
  cudaEventRecord(S().timer_start, S().stream);
}

extern "C" double cqlcuda_timer_end_ms(void)
{
  CqlState& s = S();
  cudaEventRecord(s.timer_stop, s.stream);
  if (!wait_event(s.timer_stop, "timer")) return -1.0;
  float ms = 0;
  cudaEventElapsedTime(&ms, s.timer_start, s.timer_stop);
  return ms;
}

// ---------------------------------------------------------------------------------------------
// lanes: a thread's own stream, batch, kernel arguments and pooled-buffer names

extern "C" int cqlcuda_thread_lane_begin(const char* pool_tag)
{
  CqlState& s = S();
  if (tl_lane) return 1;
  {
    std::lock_guard<std::recursive_mutex> g(s.lock);
    if (!ensure_init()) return 0;
    s.lanes_open += 1;
  }
  CqlLane* l = new CqlLane();
  l->is_main = 0;
  l->launches = 0;
  l->batch.active = 0;
  l->batch.failed = 0;
  l->batch.staging.host = nullptr;
  l->batch.staging.capacity = 0;
  l->batch.staging.used = 0;
  l->pool_tag = std::string(pool_tag ? pool_tag : "") + "/";
  if (!note_cuda(cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking), "cudaStreamCreate(lane)"))
  {
    delete l;
    std::lock_guard<std::recursive_mutex> g(s.lock);
    s.lanes_open -= 1;
    return 0;
  }
  tl_lane = l;
  return 1;
}

extern "C" void cqlcuda_thread_lane_end(void)
{
  CqlLane* l = tl_lane;
  if (!l) return;
  wait_stream(l->stream, "lane end");
  for (auto& g : l->graphs) graph_entry_free(g.second);
  l->graphs.clear();
  staging_release(l->batch.staging);
  cudaStreamDestroy(l->stream);
  tl_lane = nullptr;
  delete l;
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  if (s.lanes_open) s.lanes_open -= 1;
}

// ---------------------------------------------------------------------------------------------
// persistent kernels: an entry point of a generated kernel's module launched on a stream of its own and left
// running. It takes its work from device memory that the host fills through copies queued on the
// persistent's copy stream (they land in the order queued) and returns by itself at its idle limit; the host
// never waits on it without a time limit.

struct CqlPersistent
{
  CqlKernel* kernel;
  cudaKernel_t fn;
  cudaStream_t stream, copies;
  CqlLaunch args;
  int launched;
  uint32_t ctas;     // the grid of the last launch
};

extern "C" CqlPersistent* cqlcuda_persistent_create(CqlKernel* k, const char* entry)
{
  CqlState& s = S();
  std::lock_guard<std::recursive_mutex> g(s.lock);
  if (!ensure_init()) return nullptr;
  if (!k || !k->generated || !k->library || !entry)
  {
    set_error("cqlcuda_persistent_create: a generated kernel and an entry point name are needed");
    return nullptr;
  }
  cudaKernel_t fn = nullptr;
  if (!note_cuda(cudaLibraryGetKernel(&fn, k->library, entry), "cudaLibraryGetKernel(persistent entry)")) return nullptr;
  if (k->gen_smem > 48 * 1024) cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k->gen_smem);
  CqlPersistent* p = new CqlPersistent();
  p->kernel = k;
  p->fn = fn;
  p->launched = 0;
  p->ctas = 0;
  memset(&p->args, 0, sizeof(p->args));
  if (!note_cuda(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking), "cudaStreamCreate(persistent)"))
  {
    delete p;
    return nullptr;
  }
  if (!note_cuda(cudaStreamCreateWithFlags(&p->copies, cudaStreamNonBlocking), "cudaStreamCreate(persistent copies)"))
  {
    cudaStreamDestroy(p->stream);
    delete p;
    return nullptr;
  }
  s.persistent_open += 1;
  return p;
}

// 1 while the kernel runs, 0 once it has returned (or was never launched), -1 if it returned with an error
extern "C" int cqlcuda_persistent_running(CqlPersistent* p)
{
  if (!p || !p->launched) return 0;
  cudaError_t e = cudaStreamQuery(p->stream);
  if (e == cudaErrorNotReady) return 1;
  p->launched = 0;
  if (e != cudaSuccess)
  {
    note_cuda(e, "persistent kernel");
    return -1;
  }
  return 0;
}

// launches the entry with the kernel's arguments as this thread set them, `ctas` CTAs of the kernel's block
// size and shared memory; `zero`/`zero_bytes` (optional) is cleared on the kernel's stream first
extern "C" int cqlcuda_persistent_launch(CqlPersistent* p, uint32_t ctas, CqlBuffer* zero, uint64_t zero_bytes)
{
  if (!p) return 0;
  if (ctas == 0)
  {
    // every CTA resident at once (a CTA left waiting for a slot would hold back every item until the
    // resident ones reach their idle limit)
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)p->fn, (int)p->kernel->gen_block, p->kernel->gen_smem) != cudaSuccess ||
        per_sm < 1)
    {
      // the occupancy query may not take a library kernel handle: the same count from the kernel's registers
      // and shared memory against one SM's 64K registers, 228 KB of shared memory and 2048 threads
      cudaGetLastError();
      per_sm = 1;
      cudaFuncAttributes fa;
      if (cudaFuncGetAttributes(&fa, (const void*)p->fn) == cudaSuccess && fa.numRegs > 0)
      {
        int block = (int)p->kernel->gen_block;
        int warp_regs = ((fa.numRegs * 32 + 255) / 256) * 256;              // registers go to a warp in 256s
        int by_regs = 65536 / (warp_regs * ((block + 31) / 32));
        int by_smem = (228 * 1024) / (int)(p->kernel->gen_smem + fa.sharedSizeBytes + 1024);
        int by_threads = 2048 / block;
        per_sm = std::max(1, std::min(std::min(by_regs, by_smem), std::min(by_threads, 32)));
      }
      else cudaGetLastError();
    }
    // and one CTA's room an SM left over where four or more fit, so that other lanes' kernels still find an
    // SM while this one waits for work (with fewer, the room would cost the scan a third of its warps or more)
    if (per_sm >= 4) per_sm -= 1;
    ctas = (uint32_t)per_sm * (uint32_t)g_cql_sm_count;
  }
  if (cqlcuda_persistent_running(p) == 1)
  {
    set_error("cqlcuda_persistent_launch: the kernel is still running");
    return 0;
  }
  if (zero && !note_cuda(cudaMemsetAsync(zero->dptr, 0, std::min(zero_bytes, zero->size), p->stream), "persistent zero")) return 0;
  p->args = L().args[p->kernel];
  void* params[] = { &p->args };
  if (!note_cuda(cudaLaunchKernel((const void*)p->fn, dim3(ctas), dim3(p->kernel->gen_block), params, p->kernel->gen_smem, p->stream),
                 "persistent launch"))
    return 0;
  cql_note_launch();
  p->launched = 1;
  p->ctas = ctas;
  return 1;
}

extern "C" uint32_t cqlcuda_persistent_ctas(CqlPersistent* p) { return p ? p->ctas : 0; }

// queues a copy of host bytes into a device buffer on the copy stream; the source must stay unchanged until
// the work it describes is done
extern "C" int cqlcuda_persistent_copy(CqlPersistent* p, CqlBuffer* dst, uint64_t offset, const void* src, uint64_t size)
{
  if (!p || !dst || !src || offset > dst->size || size > dst->size - offset || dst->imported)
  {
    set_error("cqlcuda_persistent_copy: bad destination");
    return 0;
  }
  return note_cuda(cudaMemcpyAsync((char*)dst->dptr + offset, src, size, cudaMemcpyHostToDevice, p->copies), "persistent copy");
}

// waits at most timeout_ms for the kernel to return, then frees it: 1 done, 0 still running (p is kept)
extern "C" int cqlcuda_persistent_destroy(CqlPersistent* p, uint32_t timeout_ms)
{
  if (!p) return 1;
  auto t0 = std::chrono::steady_clock::now();
  while (cqlcuda_persistent_running(p) == 1)
  {
    if (std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeout_ms))
    {
      set_error("cqlcuda_persistent_destroy: the kernel still runs after %u ms", timeout_ms);
      return 0;
    }
    std::this_thread::sleep_for(std::chrono::microseconds(100));
  }
  wait_stream(p->copies, "persistent copies");
  cudaStreamDestroy(p->copies);
  cudaStreamDestroy(p->stream);
  CqlState& s = S();
  {
    std::lock_guard<std::recursive_mutex> g(s.lock);
    if (s.persistent_open) s.persistent_open -= 1;
  }
  delete p;
  return 1;
}
