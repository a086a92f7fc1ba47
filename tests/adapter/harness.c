/* Compiles the reference-side adapter files - the GPU_Backend vtable (gpu_cuda.c) and the qk_* layer
 * (query_kernel_cuda.c) - inside a translation unit laid out as the reference's unity build lays out
 * its headers (src/main.c:9-17), with the reference's own base, gpu and query_exec headers. The OS
 * layer's umbrella header is skipped (it has no Linux core or net layer); its core and net type headers
 * are included directly. Then, without a GPU:
 *   - the vtable has the size the reference's registration checks (gpu_dispatch.c:17-22) and every slot
 *     is filled;
 *   - qk_scan_source_build / qk_fused_aggregate_kernel's sources for a WHERE program built the way
 *     qe_compile_condition builds it compile with NVRTC for sm_103a, and so does qk_having_kernel's.
 * Prints one line per check; exits non-zero on the first failure. */
#define GPU_BACKEND_CUDA 1
#include "base/base_inc.h"
#define OS_INC_H
#include "os/core/os_core.h"
#include "os/net/os_net.h"
#include "thread_pool/thread_pool.h"
#include "settings/settings.h"
#include "cql/cql_inc.h"
#include "ir_gen/ir_gen_inc.h"
#include "gpu/gpu_inc.h"
#include "gpu_cuda.h"
#include "planner/plan_node.h"
#include "query_exec/query_exec.h"
#include "cqlops.h"

#include "stubs.c"
#include "gpu_cuda.c"
#include "query_kernel_cuda.c"

#define CHECK(cond, what) do { if (!(cond)) { printf("FAIL %s\n", what); return 1; } printf("ok %s\n", what); } while (0)

static U32 g_words[64];
static U32 g_consts[16];

/* `flag < 2 AND amount >= 9000.5` over flag (U32, slot 0) and amount (F64, slot 1), as the reference's
   bytecode: LoadNumCol (type << 8 | slot), PushConst index, CmpLt / CmpGe, And, Halt */
static void build_program(QE_BytecodeProgram* p)
{
  MemoryZero(p, sizeof(*p));
  U32 w[] = { QE_Opcode_LoadNumCol, (CQL_ColumnType_U32 << 8) | 0, QE_Opcode_PushConst, 0, QE_Opcode_CmpLt,
              QE_Opcode_LoadNumCol, (CQL_ColumnType_F64 << 8) | 1, QE_Opcode_PushConst, 1, QE_Opcode_CmpGe, QE_Opcode_And, QE_Opcode_Halt };
  MemoryCopy(g_words, w, sizeof(w));
  double c[2] = { 2.0, 9000.5 };
  MemoryCopy(g_consts, c, sizeof(c));
  p->words = g_words;
  p->word_count = sizeof(w) / sizeof(w[0]);
  p->consts = g_consts;
  p->const_count = 2;
  p->binding_count = 2;
  p->bindings[0].type = CQL_ColumnType_U32;
  p->bindings[0].first_slot = 0;
  p->bindings[0].slot_count = 1;
  p->bindings[1].type = CQL_ColumnType_F64;
  p->bindings[1].first_slot = 1;
  p->bindings[1].slot_count = 1;
  p->next_slot = 2;
}

int main(void)
{
  GPU_Backend* b = gpu_cuda_get_backend();
  CHECK(b->struct_size == sizeof(GPU_Backend), "struct_size is sizeof(GPU_Backend), as gpu_backend_register requires");
  int filled = 0, slots = 0;
#define SLOT(f) slots++; if (b->f) filled++; else printf("empty slot %s\n", #f);
  SLOT(init) SLOT(release) SLOT(wait) SLOT(get_executed_kernel_time_microseconds) SLOT(device_total_memory)
  SLOT(device_free_memory) SLOT(device_max_storage_buffer_range) SLOT(device_lost) SLOT(pool_begin_epoch) SLOT(memory_stats)
  SLOT(buffer_alloc) SLOT(buffer_alloc_pooled) SLOT(buffer_import_host_readonly) SLOT(buffer_import_host_readonly_pooled)
  SLOT(buffer_release) SLOT(buffer_write) SLOT(buffer_read)
  SLOT(kernel_alloc) SLOT(kernel_alloc_from_spirv) SLOT(kernel_alloc_from_spirv_spec) SLOT(generated_kernel_stats) SLOT(kernel_release)
  SLOT(kernel_execute) SLOT(kernel_set_arg_buffer) SLOT(kernel_set_arg_u64)
  SLOT(batch_begin) SLOT(batch_buffer_write) SLOT(batch_buffer_zero) SLOT(batch_buffer_fill) SLOT(batch_kernel_execute)
  SLOT(batch_buffer_read) SLOT(batch_end)
  SLOT(stream_alloc) SLOT(stream_release) SLOT(stream_slot_begin) SLOT(stream_copy) SLOT(stream_zero) SLOT(stream_fill)
  SLOT(stream_dispatch) SLOT(stream_read) SLOT(stream_submit) SLOT(stream_wait) SLOT(stream_get_stats)
  SLOT(scratch_arena) SLOT(name)
#undef SLOT
  /* every member after struct_size is one function pointer: the count above covers the whole struct */
  CHECK((sizeof(GPU_Backend) - offsetof(GPU_Backend, init)) / sizeof(void*) == (size_t)slots, "the slot list covers every member");
  CHECK(filled == slots, "every slot filled");
  String8 name = b->name();
  CHECK(name.size == 4 && memcmp(name.str, "cuda", 4) == 0, "backend name");
  CHECK(sizeof(GPU_MemoryStats) == sizeof(CqlMemoryStats), "GPU_MemoryStats and CqlMemoryStats have one layout");
  CHECK((U32)GPU_BufferFlag_ReadWrite == (U32)CQLCUDA_BUFFER_READ_WRITE && (U32)GPU_BufferFlag_Shared == (U32)CQLCUDA_BUFFER_SHARED, "buffer flag bits");

  qk_init();
  CHECK(qk_compiler_available(), "NVRTC available to the qk_* layer");
  Arena* arena = arena_alloc();
  QE_BytecodeProgram prog;
  build_program(&prog);
  QK_HybridInfo hybrid;
  MemoryZero(&hybrid, sizeof(hybrid));
  hybrid.allow = 1;
  String8 src = { 0 };
  CHECK(qk_scan_source_build(arena, &prog, &hybrid, 0, &src) && src.size > 0, "qk_scan_source_build emits a source");
  CHECK(!hybrid.is_hybrid, "hybrid requests answered with the full-width scan");
  CHECK(strstr((char*)src.str, "__global__") != 0, "the scan source is CUDA C++");
  CHECK(cqlcuda_compile_check((char*)src.str, src.size), "the scan source compiles for sm_103a");

  QK_FusedAgg fuse;
  MemoryZero(&fuse, sizeof(fuse));
  fuse.column_count = 1;
  fuse.slots[0] = 1;
  fuse.coltypes[0] = CQL_ColumnType_F64;
  String8 fsrc = { 0 };
  CHECK(qk_scan_source_build(arena, &prog, 0, &fuse, &fsrc) && fsrc.size > 0, "fused aggregate source");
  CHECK(cqlcuda_compile_check((char*)fsrc.str, fsrc.size), "the fused aggregate source compiles");
  QK_FusedAgg group;
  MemoryZero(&group, sizeof(group));
  group.grouped = 1;
  group.key_count = 1;
  group.key_slots[0] = 0;
  group.key_types[0] = CQL_ColumnType_U32;
  group.key_ranges[0] = 100;
  group.group_count = 100;
  String8 gsrc = { 0 };
  CHECK(qk_scan_source_build(arena, &prog, 0, &group, &gsrc) && gsrc.size > 0, "fused group source");
  CHECK(cqlcuda_compile_check((char*)gsrc.str, gsrc.size), "the fused group source compiles");
  CHECK(strcmp((char*)src.str, (char*)fsrc.str) != 0 && strcmp((char*)fsrc.str, (char*)gsrc.str) != 0, "three different kernels");

  /* the same program with other literals gives the same source: literals stay in binding 1 */
  double c2[2] = { 7.0, -3.25 };
  MemoryCopy(g_consts, c2, sizeof(c2));
  String8 src2 = { 0 };
  CHECK(qk_scan_source_build(arena, &prog, 0, 0, &src2) && src2.size == src.size && memcmp(src2.str, src.str, src.size) == 0,
        "literals do not change the source");

  char hsrc[8192];
  uint64_t hlen = 0;
  CHECK(cqlops_having_source("v0 > lit[0] && fabs(v1) <= lit[1]", 8, hsrc, sizeof(hsrc), &hlen), "HAVING source");
  CHECK(cqlcuda_compile_check(hsrc, hlen), "the HAVING source compiles");
  CHECK(!cqlops_having_source("system(0)", 8, hsrc, sizeof(hsrc), &hlen), "a HAVING condition outside the whitelist is refused");

  String8 n1 = qk_kernel_name(1, 2), n2 = qk_kernel_name(1, 2);
  CHECK(n1.str == n2.str && n1.size == 8 + 32, "kernel names are interned as qk_scan_<key><check>");
  CHECK(qk_sort_kernel(arena, 2, 0, 0, 0) == 0 && qk_compact_kernel(arena, 0) == 0, "precompiled-contract kernels left to the caller's fallback");
  printf("all ok\n");
  return 0;
}
