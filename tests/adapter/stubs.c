/* The base-layer, OS, settings and GPU-dispatch functions the adapter files call, for compiling them
 * against the reference's own headers outside its unity build (test infrastructure: the reference's
 * implementations need its Win32 OS layer). Arenas are plain malloc, settings take their defaults or
 * an environment variable of the same name, and gpu_kernel_alloc* forward to the CUDA backend's vtable
 * as gpu_dispatch.c forwards to the active backend. */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

internal void log_logf(LogLevel level, const char* file, int line, const char* fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  fprintf(stderr, "[log %d %s:%d] ", (int)level, file, line);
  vfprintf(stderr, fmt, ap);
  fputc('\n', stderr);
  va_end(ap);
}

internal Arena* arena_alloc_(ArenaParams* params)
{
  (void)params;
  return (Arena*)calloc(1, sizeof(Arena));
}

internal void* arena_push(Arena* arena, U64 size, U64 align)
{
  (void)arena;
  (void)align;
  return calloc(1, size ? size : 1);
}

internal String8 str8(U8* str, U64 size)
{
  String8 r;
  r.str = str;
  r.size = size;
  return r;
}

internal String8 str8_zero(void)
{
  String8 r = { 0 };
  return r;
}

internal String8 str8_cstring(char* c)
{
  return str8((U8*)c, c ? strlen(c) : 0);
}

internal U64 settings_u64(String8 key, U64 default_value)
{
  char name[128];
  U64 n = key.size < sizeof(name) - 1 ? key.size : sizeof(name) - 1;
  memcpy(name, key.str, n);
  name[n] = 0;
  const char* v = getenv(name);
  return v ? (U64)strtoull(v, 0, 10) : default_value;
}

internal OS_Handle os_handle_zero(void)
{
  OS_Handle h = { { 0, 0 } };
  return h;
}

internal B32 os_handle_match(OS_Handle a, OS_Handle b)
{
  return a.u64[0] == b.u64[0] && a.u64[1] == b.u64[1];
}

internal OS_Handle os_mutex_alloc(void)
{
  OS_Handle h = { { 1, 0 } };
  return h;
}

internal void os_mutex_take(OS_Handle mutex) { (void)mutex; }
internal void os_mutex_drop(OS_Handle mutex) { (void)mutex; }

internal GPU_Backend* gpu_cuda_get_backend(void);

internal GPU_Kernel* gpu_kernel_alloc(String8 name)
{
  return gpu_cuda_get_backend()->kernel_alloc(name);
}

internal GPU_Kernel* gpu_kernel_alloc_from_spirv(String8 name, String8 spirv)
{
  return gpu_cuda_get_backend()->kernel_alloc_from_spirv(name, spirv);
}
