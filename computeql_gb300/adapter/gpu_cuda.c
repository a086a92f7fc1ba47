/* gpu_cuda.c - GPU_Backend (src/gpu/gpu_backend.h:17-71) over libcqlcuda.so, for ComputeQL's C99
 * unity build (src/gpu/cuda/gpu_cuda.c in the reference's tree, included from gpu_inc.c when
 * GPU_BACKEND_CUDA is set).
 *
 * Every slot forwards to the cqlcuda_* function of the same name (include/cqlcuda.h). The handle types
 * are opaque on both sides, GPU_BufferFlags has the CQLCUDA_BUFFER_* bit values and GPU_MemoryStats the
 * CqlMemoryStats field order, so arguments pass through unchanged. The operator layer's failure hooks
 * (g_gpu_fault_alloc_at, g_gpu_evict_hook, src/gpu/gpu.h:68,111-113) are globals it may set at any
 * time; they are handed to the backend before each allocation.
 */

internal void gpu_cuda_init(void)
{
  if (!cqlcuda_init()) log_error("gpu_cuda: %s", cqlcuda_last_error());
}
internal void gpu_cuda_release(void) { cqlcuda_release(); }
internal void gpu_cuda_wait(void) { cqlcuda_wait(); }
internal U64 gpu_cuda_kernel_us(void) { return cqlcuda_get_executed_kernel_time_microseconds(); }
internal U64 gpu_cuda_total(void) { return cqlcuda_device_total_memory(); }
internal U64 gpu_cuda_free(void) { return cqlcuda_device_free_memory(); }
internal U64 gpu_cuda_range(void) { return cqlcuda_device_max_storage_buffer_range(); }
internal B32 gpu_cuda_lost(void) { return cqlcuda_device_lost() ? 1 : 0; }
internal void gpu_cuda_epoch(void) { cqlcuda_pool_begin_epoch(); }

internal GPU_MemoryStats gpu_cuda_mem_stats(void)
{
  CqlMemoryStats s = cqlcuda_memory_stats();
  GPU_MemoryStats r;
  r.bytes_in_use = s.bytes_in_use;
  r.bytes_peak = s.bytes_peak;
  r.alloc_failures = s.alloc_failures;
  r.alloc_retry_successes = s.alloc_retry_successes;
  r.pool_evictions = s.pool_evictions;
  r.pool_evicted_bytes = s.pool_evicted_bytes;
  r.alloc_calls = s.alloc_calls;
  r.unrecovered_alloc_failures = s.unrecovered_alloc_failures;
  return r;
}

internal void gpu_cuda_sync_hooks(void)
{
  cqlcuda_set_fault_alloc_at(g_gpu_fault_alloc_at);
  cqlcuda_set_evict_hook((CqlEvictHook)g_gpu_evict_hook);
}

internal GPU_Buffer* gpu_cuda_alloc(U64 size, GPU_BufferFlags flags, void* data)
{
  gpu_cuda_sync_hooks();
  return (GPU_Buffer*)cqlcuda_buffer_alloc(size, (U32)flags, data);
}
internal GPU_Buffer* gpu_cuda_alloc_pooled(String8 name, U64 size, GPU_BufferFlags flags, void* data)
{
  gpu_cuda_sync_hooks();
  return (GPU_Buffer*)cqlcuda_buffer_alloc_pooled((const char*)name.str, name.size, size, (U32)flags, data);
}
internal GPU_Buffer* gpu_cuda_import(void* host_ptr, U64 size)
{
  return (GPU_Buffer*)cqlcuda_buffer_import_host_readonly(host_ptr, size);
}
internal GPU_Buffer* gpu_cuda_import_pooled(String8 name, void* host_ptr, U64 size)
{
  return (GPU_Buffer*)cqlcuda_buffer_import_host_readonly_pooled((const char*)name.str, name.size, host_ptr, size);
}
internal void gpu_cuda_buffer_release(GPU_Buffer* b) { cqlcuda_buffer_release((CqlBuffer*)b); }
internal void gpu_cuda_buffer_write(GPU_Buffer* b, void* data, U64 size) { cqlcuda_buffer_write((CqlBuffer*)b, data, size); }
internal void gpu_cuda_buffer_read(GPU_Buffer* b, void* data, U64 size) { cqlcuda_buffer_read((CqlBuffer*)b, data, size); }

/* kernel_alloc_from_spirv: under this backend the image is CUDA C++ source (compiled by NVRTC for
   sm_103a and cached by name) or a cubin; an empty image only looks the name up (src/gpu/gpu.h:129-130) */
internal GPU_Kernel* gpu_cuda_kernel_alloc(String8 name)
{
  return (GPU_Kernel*)cqlcuda_kernel_alloc((const char*)name.str, name.size);
}
internal GPU_Kernel* gpu_cuda_kernel_image(String8 name, String8 image)
{
  return (GPU_Kernel*)cqlcuda_kernel_alloc_from_image((const char*)name.str, name.size, image.str, image.size);
}
internal GPU_Kernel* gpu_cuda_kernel_image_spec(String8 name, String8 image, U32* spec_values, U32 spec_count)
{
  return (GPU_Kernel*)cqlcuda_kernel_alloc_from_image_spec((const char*)name.str, name.size, image.str, image.size, spec_values, spec_count);
}
internal void gpu_cuda_generated_stats(U64* out_compiles, U64* out_evictions)
{
  uint64_t c = 0, e = 0;
  cqlcuda_generated_kernel_stats(&c, &e);
  if (out_compiles) *out_compiles = c;
  if (out_evictions) *out_evictions = e;
}
internal void gpu_cuda_kernel_release(GPU_Kernel* k) { cqlcuda_kernel_release((CqlKernel*)k); }
internal void gpu_cuda_kernel_execute(GPU_Kernel* k, U32 gws, U32 lws) { cqlcuda_kernel_execute((CqlKernel*)k, gws, lws); }
internal void gpu_cuda_arg_buffer(GPU_Kernel* k, U32 index, GPU_Buffer* b) { cqlcuda_kernel_set_arg_buffer((CqlKernel*)k, index, (CqlBuffer*)b); }
internal void gpu_cuda_arg_u64(GPU_Kernel* k, U32 index, U64 value) { cqlcuda_kernel_set_arg_u64((CqlKernel*)k, index, value); }

internal GPU_Batch* gpu_cuda_batch_begin(U64 up, U64 down) { return (GPU_Batch*)cqlcuda_batch_begin(up, down); }
internal void gpu_cuda_batch_write(GPU_Batch* b, GPU_Buffer* x, void* d, U64 n) { cqlcuda_batch_buffer_write((CqlBatch*)b, (CqlBuffer*)x, d, n); }
internal void gpu_cuda_batch_zero(GPU_Batch* b, GPU_Buffer* x, U64 n) { cqlcuda_batch_buffer_zero((CqlBatch*)b, (CqlBuffer*)x, n); }
internal void gpu_cuda_batch_fill(GPU_Batch* b, GPU_Buffer* x, U64 n, U32 v) { cqlcuda_batch_buffer_fill((CqlBatch*)b, (CqlBuffer*)x, n, v); }
internal void gpu_cuda_batch_execute(GPU_Batch* b, GPU_Kernel* k, U32 gws, U32 lws) { cqlcuda_batch_kernel_execute((CqlBatch*)b, (CqlKernel*)k, gws, lws); }
internal void gpu_cuda_batch_read(GPU_Batch* b, GPU_Buffer* x, void* d, U64 n) { cqlcuda_batch_buffer_read((CqlBatch*)b, (CqlBuffer*)x, d, n); }
internal B32 gpu_cuda_batch_end(GPU_Batch* b) { return cqlcuda_batch_end((CqlBatch*)b) ? 1 : 0; }

internal GPU_Stream* gpu_cuda_stream_alloc(U32 slots) { return (GPU_Stream*)cqlcuda_stream_alloc(slots); }
internal void gpu_cuda_stream_release(GPU_Stream* s) { cqlcuda_stream_release((CqlStream*)s); }
internal B32 gpu_cuda_stream_slot_begin(GPU_Stream* s, U32 slot, U64 up, U64 down) { return cqlcuda_stream_slot_begin((CqlStream*)s, slot, up, down) ? 1 : 0; }
internal B32 gpu_cuda_stream_copy(GPU_Stream* s, U32 slot, GPU_Buffer* dst, void* host, U64 n) { return cqlcuda_stream_copy((CqlStream*)s, slot, (CqlBuffer*)dst, host, n) ? 1 : 0; }
internal void gpu_cuda_stream_zero(GPU_Stream* s, U32 slot, GPU_Buffer* b, U64 n) { cqlcuda_stream_zero((CqlStream*)s, slot, (CqlBuffer*)b, n); }
internal void gpu_cuda_stream_fill(GPU_Stream* s, U32 slot, GPU_Buffer* b, U64 n, U32 v) { cqlcuda_stream_fill((CqlStream*)s, slot, (CqlBuffer*)b, n, v); }
internal void gpu_cuda_stream_dispatch(GPU_Stream* s, U32 slot, GPU_Kernel* k, U32 gws, U32 lws) { cqlcuda_stream_dispatch((CqlStream*)s, slot, (CqlKernel*)k, gws, lws); }
internal void gpu_cuda_stream_read(GPU_Stream* s, U32 slot, GPU_Buffer* b, void* d, U64 n) { cqlcuda_stream_read((CqlStream*)s, slot, (CqlBuffer*)b, d, n); }
internal B32 gpu_cuda_stream_submit(GPU_Stream* s, U32 slot) { return cqlcuda_stream_submit((CqlStream*)s, slot) ? 1 : 0; }
internal B32 gpu_cuda_stream_wait(GPU_Stream* s, U32 slot) { return cqlcuda_stream_wait((CqlStream*)s, slot) ? 1 : 0; }
internal GPU_StreamStats gpu_cuda_stream_stats(GPU_Stream* s)
{
  CqlStreamStats c = cqlcuda_stream_get_stats((CqlStream*)s);
  GPU_StreamStats r;
  r.bytes_copied = c.bytes_copied;
  r.imports_created = c.imports_created;
  r.import_microseconds = c.import_microseconds;
  r.staged_bytes = c.staged_bytes;
  r.separate_copy_queue = c.separate_copy_queue ? 1 : 0;
  return r;
}

global Arena* g_gpu_cuda_scratch = 0;
internal Arena* gpu_cuda_scratch_arena(void)
{
  if (!g_gpu_cuda_scratch) g_gpu_cuda_scratch = arena_alloc();
  return g_gpu_cuda_scratch;
}
internal String8 gpu_cuda_name(void) { return str8_lit("cuda"); }

internal GPU_Backend*
gpu_cuda_get_backend(void)
{
  local_persist GPU_Backend b;
  b.struct_size = (U32)sizeof(GPU_Backend);
  b.init = gpu_cuda_init;
  b.release = gpu_cuda_release;
  b.wait = gpu_cuda_wait;
  b.get_executed_kernel_time_microseconds = gpu_cuda_kernel_us;
  b.device_total_memory = gpu_cuda_total;
  b.device_free_memory = gpu_cuda_free;
  b.device_max_storage_buffer_range = gpu_cuda_range;
  b.device_lost = gpu_cuda_lost;
  b.pool_begin_epoch = gpu_cuda_epoch;
  b.memory_stats = gpu_cuda_mem_stats;
  b.buffer_alloc = gpu_cuda_alloc;
  b.buffer_alloc_pooled = gpu_cuda_alloc_pooled;
  b.buffer_import_host_readonly = gpu_cuda_import;
  b.buffer_import_host_readonly_pooled = gpu_cuda_import_pooled;
  b.buffer_release = gpu_cuda_buffer_release;
  b.buffer_write = gpu_cuda_buffer_write;
  b.buffer_read = gpu_cuda_buffer_read;
  b.kernel_alloc = gpu_cuda_kernel_alloc;
  b.kernel_alloc_from_spirv = gpu_cuda_kernel_image;
  b.kernel_alloc_from_spirv_spec = gpu_cuda_kernel_image_spec;
  b.generated_kernel_stats = gpu_cuda_generated_stats;
  b.kernel_release = gpu_cuda_kernel_release;
  b.kernel_execute = gpu_cuda_kernel_execute;
  b.kernel_set_arg_buffer = gpu_cuda_arg_buffer;
  b.kernel_set_arg_u64 = gpu_cuda_arg_u64;
  b.batch_begin = gpu_cuda_batch_begin;
  b.batch_buffer_write = gpu_cuda_batch_write;
  b.batch_buffer_zero = gpu_cuda_batch_zero;
  b.batch_buffer_fill = gpu_cuda_batch_fill;
  b.batch_kernel_execute = gpu_cuda_batch_execute;
  b.batch_buffer_read = gpu_cuda_batch_read;
  b.batch_end = gpu_cuda_batch_end;
  b.stream_alloc = gpu_cuda_stream_alloc;
  b.stream_release = gpu_cuda_stream_release;
  b.stream_slot_begin = gpu_cuda_stream_slot_begin;
  b.stream_copy = gpu_cuda_stream_copy;
  b.stream_zero = gpu_cuda_stream_zero;
  b.stream_fill = gpu_cuda_stream_fill;
  b.stream_dispatch = gpu_cuda_stream_dispatch;
  b.stream_read = gpu_cuda_stream_read;
  b.stream_submit = gpu_cuda_stream_submit;
  b.stream_wait = gpu_cuda_stream_wait;
  b.stream_get_stats = gpu_cuda_stream_stats;
  b.scratch_arena = gpu_cuda_scratch_arena;
  b.name = gpu_cuda_name;
  return &b;
}
