/*
 * cqlcuda.h - C ABI of the GB300 (sm_103a) execution backend for ComputeQL's GPU operators.
 *
 * Every entry point here replaces one function pointer of the reference's backend vtable
 * `GPU_Backend` (src/gpu/gpu_backend.h:17-71) or one forwarder of the backend-neutral API
 * (src/gpu/gpu.h:95-159). The reference's operator layer (src/query_exec) keeps calling
 * gpu_* functions; a C99 adapter, computeql_gb300/adapter/gpu_cuda.c (src/gpu/cuda/gpu_cuda.c in
 * the reference's tree), fills the vtable with these functions. Types are plain C: opaque handles,
 * pointers and sizes, no CUDA or torch types.
 *
 * Kernels are looked up by the names of the reference's shaders (src/gpu/vulkan/shaders/<name>.comp)
 * and honour the same binding contract: up to 16 buffer bindings and 8 U64 push-constant slots,
 * seen by the kernel as 16 32-bit words, low word first (src/gpu/vulkan/gpu_vulkan.h:6-9).
 * A kernel is free to pick its own grid: `global_work_size`/`local_work_size` are accepted for
 * contract compatibility, and each kernel writes exactly the outputs its shader writes, with
 * entries the shader would leave for workgroups it did not launch filled with neutral values.
 *
 * Errors follow the reference: allocation failure returns NULL, a failed batch or stream wait
 * returns 0, a sticky device-lost flag is raised on unrecoverable CUDA errors, and the text of
 * the last error is available from cqlcuda_last_error().
 */
#ifndef CQLCUDA_H
#define CQLCUDA_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CQLCUDA_MAX_BINDINGS 16
#define CQLCUDA_PUSH_SLOTS   8

/* Buffer flags, bit-for-bit the reference's GPU_BufferFlags (src/gpu/gpu.h:8-22). */
enum
{
  CQLCUDA_BUFFER_READ              = 1u << 0,
  CQLCUDA_BUFFER_WRITE             = 1u << 1,
  CQLCUDA_BUFFER_READ_WRITE        = 1u << 2,
  CQLCUDA_BUFFER_HOST_VISIBLE      = 1u << 3,
  CQLCUDA_BUFFER_DEVICE_LOCAL      = 1u << 4,
  CQLCUDA_BUFFER_HOST_CACHED       = 1u << 5,
  CQLCUDA_BUFFER_ZERO_COPY         = 1u << 6,
  CQLCUDA_BUFFER_COPY_HOST_POINTER = 1u << 7,
  CQLCUDA_BUFFER_DYNAMIC           = 1u << 8,
  CQLCUDA_BUFFER_SHARED            = 1u << 9,
};

typedef struct CqlBuffer CqlBuffer;
typedef struct CqlKernel CqlKernel;
typedef struct CqlBatch  CqlBatch;
typedef struct CqlStream CqlStream;

/* Same fields and order as GPU_MemoryStats (src/gpu/gpu.h:24-35). */
typedef struct CqlMemoryStats
{
  uint64_t bytes_in_use;
  uint64_t bytes_peak;
  uint64_t alloc_failures;
  uint64_t alloc_retry_successes;
  uint64_t pool_evictions;
  uint64_t pool_evicted_bytes;
  uint64_t alloc_calls;
  uint64_t unrecovered_alloc_failures;
} CqlMemoryStats;

/* Same fields and order as GPU_StreamStats (src/gpu/gpu.h:87-94). */
typedef struct CqlStreamStats
{
  uint64_t bytes_copied;
  uint64_t imports_created;
  uint64_t import_microseconds;
  uint64_t staged_bytes;
  uint32_t separate_copy_queue;
} CqlStreamStats;

/* Eviction hook: GPU_EvictHook (src/gpu/gpu.h:111-113). Called with the bytes still wanted after
   pooled buffers were evicted; returns the bytes it freed. */
typedef uint64_t (*CqlEvictHook)(uint64_t bytes_wanted);

/* ---- device (GPU_Backend init/release/wait/... gpu_backend.h:21-30) ---- */
int      cqlcuda_init(void);                                   /* gpu_backend.h:21 init; returns 1 on success */
void     cqlcuda_release(void);                                /* gpu_backend.h:22 release */
void     cqlcuda_wait(void);                                   /* gpu_backend.h:23 wait */
uint64_t cqlcuda_get_executed_kernel_time_microseconds(void);  /* gpu_backend.h:24 */
uint64_t cqlcuda_device_total_memory(void);                    /* gpu_backend.h:25 */
uint64_t cqlcuda_device_free_memory(void);                     /* gpu_backend.h:26 */
uint64_t cqlcuda_device_max_storage_buffer_range(void);        /* gpu_backend.h:27 */
int      cqlcuda_device_lost(void);                            /* gpu_backend.h:28 */
void     cqlcuda_pool_begin_epoch(void);                       /* gpu_backend.h:29 */
/* Frees pooled buffers not used in the current epoch, least recently used first, until `bytes_wanted`
   are freed (UINT64_MAX: all of them); returns the bytes freed. gpu_vulkan_pool_evict
   (src/gpu/vulkan/gpu_vulkan.c:1577-1617), which the reference's failure tests call to start each run
   cold (src/tests/bench_alloc_fault.c:236-241). Does nothing while a batch is open or a lane is open. */
uint64_t cqlcuda_pool_evict(uint64_t bytes_wanted);
CqlMemoryStats cqlcuda_memory_stats(void);                     /* gpu_backend.h:30 */
uint32_t cqlcuda_sm_count(void);                               /* device property the kernels size grids by */

/* ---- buffers (gpu_backend.h:32-38) ---- */
CqlBuffer* cqlcuda_buffer_alloc(uint64_t size, uint32_t flags, const void* data);                       /* :32 */
CqlBuffer* cqlcuda_buffer_alloc_pooled(const char* name, uint64_t name_len, uint64_t size,
                                       uint32_t flags, const void* data);                             /* :33 */
CqlBuffer* cqlcuda_buffer_import_host_readonly(const void* host_ptr, uint64_t size);                   /* :34 */
CqlBuffer* cqlcuda_buffer_import_host_readonly_pooled(const char* name, uint64_t name_len,
                                                      const void* host_ptr, uint64_t size);           /* :35 */
void       cqlcuda_buffer_release(CqlBuffer* buffer);                                                  /* :36 */
void       cqlcuda_buffer_write(CqlBuffer* buffer, const void* data, uint64_t size);                   /* :37 */
void       cqlcuda_buffer_read(CqlBuffer* buffer, void* data, uint64_t size);                          /* :38 */
uint64_t   cqlcuda_buffer_size(const CqlBuffer* buffer);       /* the bound range a kernel sees (VkDescriptorBufferInfo.range, gpu_vulkan.c:2797) */
void*      cqlcuda_buffer_device_pointer(const CqlBuffer* buffer); /* for zero-copy interop (DLPack/torch) by host code */

/* ---- kernels (gpu_backend.h:40-47) ---- */
CqlKernel* cqlcuda_kernel_alloc(const char* name, uint64_t name_len);                                  /* :40, by shader name */
/* :41 kernel_alloc_from_spirv. The reference hands over SPIR-V; here `image` is CUDA C++ source
   (compiled with NVRTC for sm_103a) or a cubin. An empty image only looks the name up. */
CqlKernel* cqlcuda_kernel_alloc_from_image(const char* name, uint64_t name_len, const void* image, uint64_t image_len);
CqlKernel* cqlcuda_kernel_alloc_from_image_spec(const char* name, uint64_t name_len, const void* image, uint64_t image_len,
                                                const uint32_t* spec_values, uint32_t spec_count);    /* :42 */
void       cqlcuda_generated_kernel_stats(uint64_t* out_compiles, uint64_t* out_evictions);            /* :43 */
/* Generated (NVRTC) kernels kept loaded: the reference's GPU_VULKAN_MAX_GENERATED_KERNELS (default 64, at
   least 8, src/gpu/vulkan/gpu_vulkan.c:75). Past the cap the least recently looked-up generated kernel is
   unloaded and counted as an eviction (gpu_vulkan.c:2721-2737), after the GPU drains and with every plan
   graph that launches it; the 8 most recently looked-up are kept, and nothing is evicted while the main
   lane's batch is open. A handle to an evicted kernel stays valid: its dispatch fails with an error, and a
   new lookup by name (with its source) compiles it again. */
void       cqlcuda_set_generated_kernel_cap(uint32_t cap);
void       cqlcuda_kernel_release(CqlKernel* kernel);                                                  /* :44, kernels are cached: no-op */
void       cqlcuda_kernel_execute(CqlKernel* kernel, uint32_t global_work_size, uint32_t local_work_size); /* :45, synchronous */
void       cqlcuda_kernel_set_arg_buffer(CqlKernel* kernel, uint32_t index, CqlBuffer* buffer);        /* :46 */
void       cqlcuda_kernel_set_arg_u64(CqlKernel* kernel, uint32_t index, uint64_t value);              /* :47 */
/* Binding at a byte offset into a buffer: a chunk of a resident column without a copy. Not in the
   reference vtable; the adapter uses offset 0. */
void       cqlcuda_kernel_set_arg_buffer_range(CqlKernel* kernel, uint32_t index, CqlBuffer* buffer, uint64_t offset, uint64_t size);

/* ---- batches (gpu_backend.h:49-55) ---- */
CqlBatch* cqlcuda_batch_begin(uint64_t upload_bytes_needed, uint64_t download_bytes_needed);           /* :49 */
void      cqlcuda_batch_buffer_write(CqlBatch* batch, CqlBuffer* buffer, const void* data, uint64_t size); /* :50 */
void      cqlcuda_batch_buffer_zero(CqlBatch* batch, CqlBuffer* buffer, uint64_t size);                 /* :51 */
void      cqlcuda_batch_buffer_fill(CqlBatch* batch, CqlBuffer* buffer, uint64_t size, uint32_t value);  /* :52 */
void      cqlcuda_batch_kernel_execute(CqlBatch* batch, CqlKernel* kernel, uint32_t global_work_size, uint32_t local_work_size); /* :53 */
void      cqlcuda_batch_buffer_read(CqlBatch* batch, CqlBuffer* buffer, void* out_data, uint64_t size);  /* :54 */
/* The same from byte `offset` of the buffer (no reference counterpart: a read of one word of a device
   array, such as the total a prefix sum leaves after its last element). */
void      cqlcuda_batch_buffer_read_at(CqlBatch* batch, CqlBuffer* buffer, uint64_t offset, void* out_data, uint64_t size);
/* cqlcuda_batch_buffer_fill from byte `offset` (a multiple of 4) of the buffer (no reference counterpart:
   several output arrays of one operator kept in one buffer). */
void      cqlcuda_batch_fill_range(CqlBatch* batch, CqlBuffer* buffer, uint64_t offset, uint64_t size, uint32_t value);
int       cqlcuda_batch_end(CqlBatch* batch);                                                            /* :55, 0 on failure (reads zero-filled) */
/* A batch for a plan shape (no reference counterpart): its writes, fills, dispatches and reads are
   recorded, and at cqlcuda_batch_end the record runs as a CUDA graph - the one captured the second time a
   batch of the same shape ended (the same operations on the same buffers with the same kernel arguments;
   only the bytes written may differ), replayed with the new bytes in one launch; a shape met once runs as
   an ordinary batch. Only the main lane keeps graphs (up to 32); on a thread's own lane this opens an
   ordinary batch. A record that cannot be captured, and any record while kernel profiling is on (its kernels are
   timed one by one), runs as an ordinary batch. plan_key tells shapes apart. */
CqlBatch* cqlcuda_batch_begin_graph(uint64_t upload_bytes_needed, uint64_t download_bytes_needed, uint64_t plan_key);
/* On (the default) or off: with graphs off, plan-shape batches run as ordinary batches. */
void      cqlcuda_graph_enable(int on);
/* Graphs captured, replayed, and records that ran without one, since start. */
void      cqlcuda_graph_stats(uint64_t* out_captures, uint64_t* out_replays, uint64_t* out_fallbacks);

/* ---- streams (gpu_backend.h:57-67) ---- */
CqlStream* cqlcuda_stream_alloc(uint32_t slot_count);                                                    /* :57, 1..8 slots */
void       cqlcuda_stream_release(CqlStream* stream);                                                    /* :58 */
int        cqlcuda_stream_slot_begin(CqlStream* stream, uint32_t slot, uint64_t upload_bytes, uint64_t readback_bytes); /* :59 */
int        cqlcuda_stream_copy(CqlStream* stream, uint32_t slot, CqlBuffer* destination, const void* host_ptr, uint64_t size); /* :60 */
void       cqlcuda_stream_zero(CqlStream* stream, uint32_t slot, CqlBuffer* buffer, uint64_t size);      /* :61 */
void       cqlcuda_stream_fill(CqlStream* stream, uint32_t slot, CqlBuffer* buffer, uint64_t size, uint32_t value); /* :62 */
void       cqlcuda_stream_dispatch(CqlStream* stream, uint32_t slot, CqlKernel* kernel, uint32_t global_work_size, uint32_t local_work_size); /* :63 */
void       cqlcuda_stream_read(CqlStream* stream, uint32_t slot, CqlBuffer* buffer, void* out_data, uint64_t size); /* :64 */
int        cqlcuda_stream_submit(CqlStream* stream, uint32_t slot);                                      /* :65 */
int        cqlcuda_stream_wait(CqlStream* stream, uint32_t slot);                                        /* :66, bounded wait */
CqlStreamStats cqlcuda_stream_get_stats(CqlStream* stream);                                              /* :67 */

/* ---- failure injection, eviction hook, kernel log and profile (src/gpu/gpu.h:38-113) ---- */
void     cqlcuda_set_fault_alloc_at(uint64_t call_index);     /* g_gpu_fault_alloc_at (gpu.h:68): the k-th allocation call fails, 0 = off */
void     cqlcuda_set_evict_hook(CqlEvictHook hook);           /* g_gpu_evict_hook (gpu.h:111-113) */
void     cqlcuda_kernel_profile_enable(int enabled);          /* g_gpu_kernel_profile.enabled (gpu.h:48-58) */
void     cqlcuda_kernel_profile_reset(void);                  /* gpu_kernel_profile_reset (gpu.h:61) */
/* Profile entry i: its kernel name, total GPU nanoseconds and dispatch count. Returns 0 past the end. */
int      cqlcuda_kernel_profile_entry(uint32_t index, const char** out_name, uint64_t* out_total_ns, uint64_t* out_dispatches);
/* While the kernel profile is on: batches ended since the last profile reset and their host-side time in
   nanoseconds - from opening to end, waiting for the device, copying staged results to the callers. */
void     cqlcuda_host_profile(uint64_t* out_batches, uint64_t* out_open_ns, uint64_t* out_wait_ns, uint64_t* out_copy_ns);
uint32_t cqlcuda_kernel_launch_count(void);                   /* launches of this library's kernels since init */
const char* cqlcuda_last_error(void);                         /* text of the last error, "" when none */
void     cqlcuda_clear_error(void);
/* Seconds a stream or batch wait polls before it gives up and reports failure (the reference's
   30 s stream timeout, src/gpu/vulkan/gpu_vulkan.h:235). */
void     cqlcuda_set_wait_timeout_ms(uint32_t milliseconds);

/* ---- NVRTC (the shaderc replacement behind kernel_alloc_from_spirv, src/query_exec/query_kernel.c:294-457) ---- */
/* Disk cache directory for compiled cubins (empty = memory only). */
void     cqlcuda_set_module_cache_dir(const char* path);
/* Test hook mirroring QE_TEST_FAIL_SHADERC (src/query_exec/query_kernel.h:21-24): every n-th compile fails, 0 = off. */
void     cqlcuda_set_fail_compile_every(uint32_t n);
const char* cqlcuda_last_compile_log(void);
/* Compiles CUDA C++ source with NVRTC for sm_103a without loading it (no device needed): 1 when it
   compiles. The log goes to cqlcuda_last_compile_log(). */
int      cqlcuda_compile_check(const char* source, uint64_t source_len);

/* ---- slot compaction without allocation (no counterpart in the reference) ----
   For callers that cannot allocate device memory while they run a query, e.g. a serving loop that
   reserves all of HBM ahead of time for resident tables and per-query budgets, where a cudaMalloc on
   the query path can fail or force an eviction mid-query. It runs the three aggregate_compact passes
   over caller-owned device buffers and keeps the kernel's scratch (the block totals) in a static
   device array, so it calls no cudaMalloc, cudaFree or allocating library routine.
   Inputs: slot_counts/slot_owner, slot_count entries each. Outputs: slot_group (slot_count + 1
   entries: the dense group id of every occupied slot, the group total last), group_owner and
   group_count (up to slot_count entries), and *out_group_total on the host.
   Limit: slot_count <= 2^24 (256 KB of scratch, held by every GPU that loads the library until exit).
   cqlcuda_init looks the scratch address up and loads the kernel for the device it opens; on any other
   device the first call does that set-up, with that device current: make it before any stream capture.
   All calls share the scratch; calls whose work overlaps on the GPU race.
   `stream` is a cudaStream_t (NULL = the legacy default stream); the call returns once it is done.
   Returns 1, or -1 slot_count is 0 or over the limit, -2 a NULL pointer, -3 no usable device,
   -4 a launch or copy failed; cqlcuda_last_error() then says which. */
int      cqlcuda_compact_slots_noalloc(const uint32_t* slot_counts, const uint32_t* slot_owner, uint32_t slot_count,
                                       uint32_t* slot_group, uint32_t* group_owner, uint32_t* group_count, uint32_t* out_group_total,
                                       void* stream);

/* ---- raw device helpers used by the bench and tests (not in the reference vtable) ---- */
/* Fills `rows` rows of a u32 column from the splitmix64 stream seeded `seed`: row r takes draw
   r*draws_per_row + draw_index (0-based) and stores draw % range (range 0 = the full 32 bits). */
int      cqlcuda_fill_splitmix_u32(CqlBuffer* buffer, uint64_t rows, uint64_t seed, uint32_t draws_per_row, uint32_t draw_index, uint64_t range);
/* Lanes (no reference counterpart): the calling thread gets its own stream, batch, kernel arguments and
   pooled-buffer namespace (pool_tag), so several threads can run operators on the device at once.
   Without a lane a thread uses the main lane: one batch at a time, as the reference's single queue.
   Pooled buffers are not evicted while any lane is open. */
int      cqlcuda_thread_lane_begin(const char* pool_tag);
void     cqlcuda_thread_lane_end(void);
/* Fills value[r] = first + r for r < rows. */
int      cqlcuda_fill_sequence_u32(CqlBuffer* buffer, uint64_t rows, uint32_t first);
/* Fills value[r] = (r * mul + add) % modulus for r < rows, in 64-bit arithmetic, truncated to 32 bits
   (modulus 0: no reduction). The closed-form columns of the reference's scale test
   (src/tests/scale/bench_select_scale.c:38-56: region = r % 50, amount = r % 10000,
   needle_key = r * 2654435761 mod 2^32) are such fills. */
int      cqlcuda_fill_affine_u32(CqlBuffer* buffer, uint64_t rows, uint64_t mul, uint64_t add, uint64_t modulus);
/* Page-locked host memory for uploads (the reference's host-visible staging, GPU_BufferFlag_HostVisible):
   large pages where offered, on the host NUMA node nearest the GPU, registered with the device so copies
   from it run at the link's rate. NULL on failure; free with cqlcuda_host_free. */
void*    cqlcuda_host_alloc(uint64_t bytes);
void     cqlcuda_host_free(void* host_ptr);
/* Page-locked host memory mapped into the device's address space and owned by the buffer (freed with
   cqlcuda_buffer_release): kernels write answers there that the host reads through *out_host without a copy.
   Not a source or destination of cqlcuda_buffer_write/read. */
CqlBuffer* cqlcuda_buffer_alloc_host_mapped(uint64_t size, void** out_host);
/* Persistent kernels (no reference counterpart; the reference launches every shared scan anew): the entry
   point `entry` of generated kernel k's module, launched on a stream of its own and left running. It takes
   its work from device memory that the host fills with cqlcuda_persistent_copy (copies land in the order
   queued) and returns by itself at its own idle limit; no generated kernel is evicted while one exists.
   launch: with k's arguments as this thread set them, `ctas` CTAs of k's block size and shared memory (0:
   as many as are resident at once, less one CTA's room an SM for other kernels where four or more fit),
   after clearing zero_bytes of `zero` (optional) on the kernel's stream; refused while the kernel runs.
   running: 1 while it runs, 0 once it has returned, -1 if it returned with an error.
   copy: the source must stay unchanged until the work it describes is done.
   destroy: waits at most timeout_ms for the kernel to return; 0 if it still runs (p is kept). */
typedef struct CqlPersistent CqlPersistent;
CqlPersistent* cqlcuda_persistent_create(CqlKernel* k, const char* entry);
int      cqlcuda_persistent_launch(CqlPersistent* p, uint32_t ctas, CqlBuffer* zero, uint64_t zero_bytes);
int      cqlcuda_persistent_running(CqlPersistent* p);
int      cqlcuda_persistent_copy(CqlPersistent* p, CqlBuffer* dst, uint64_t offset, const void* src, uint64_t size);
int      cqlcuda_persistent_destroy(CqlPersistent* p, uint32_t timeout_ms);
uint32_t cqlcuda_persistent_ctas(CqlPersistent* p);    /* the grid of the last launch */
/* Writes `bytes` bytes of a scratch buffer, to evict the L2 between timed runs. */
int      cqlcuda_flush_l2(uint64_t bytes);
/* CUDA-event timing of everything the library enqueues between begin and end, on its own stream. */
void     cqlcuda_timer_begin(void);
double   cqlcuda_timer_end_ms(void);

#ifdef __cplusplus
}
#endif

#endif /* CQLCUDA_H */
