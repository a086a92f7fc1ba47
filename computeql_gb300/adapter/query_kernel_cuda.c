/* query_kernel_cuda.c - the per-query kernel layer of ComputeQL's operator layer (every qk_* function of
 * src/query_exec/query_kernel.h:198-240) for the GB300 CUDA backend. It takes the place of
 * query_kernel.c, which query_exec.c includes at its end (src/query_exec/query_exec.c:15358), when
 * GPU_BACKEND_CUDA is set. The header, its settings and its state (g_qk_state) stay the reference's.
 *
 * What changes is the language of the generated kernels and the compiler: a WHERE program becomes CUDA
 * C++ (cqlops_program_source, include/cqlops.h), handed to gpu_kernel_alloc_from_spirv as the kernel's
 * image, which this backend compiles with NVRTC for sm_103a and caches by name in memory and on disk.
 * The kernel naming (qk_scan_<key><check> from two hashes of the source), the failed-source memo and
 * the test hooks QE_TEST_FAIL_SHADERC and QE_TEST_KEY_BITS keep the reference's meaning.
 *
 * Per function:
 *   qk_scan_kernel, qk_scan_source_build   generated: scan_filter.comp's bindings (a hybrid request is
 *                                          answered with is_hybrid = 0: the generated scan reads every
 *                                          column it compares at full width)
 *   qk_fused_aggregate_kernel              generated: QK_FusedAgg's fused and grouped layouts
 *   qk_having_kernel                       generated: one group a thread, keep[i] (cqlops_having_source)
 *   qk_simple_kernel                       the backend's scan_simple, which reads the column, type and
 *                                          operator of every leaf from the leaf words at run time
 *   qk_join_build_kernel, qk_join_probe_hash_kernel, qk_join_probe_native_kernel, qk_hash_assign_kernel,
 *   qk_member_reduce_kernel, qk_compact_kernel, qk_hash_reduce_kernel, qk_gather_kernel
 *                                          0: the caller then takes the precompiled kernel of the same
 *                                          contract by name (hash_join_build_count, hash_join_probe,
 *                                          join_probe_native, aggregate_assign, aggregate_reduce,
 *                                          aggregate_compact, aggregate_hash_reduce_fixed,
 *                                          selection_gather), which this backend implements with every
 *                                          variant chosen from its push constants
 *   qk_sort_kernel, qk_window_flags_kernel 0: ORDER BY and window ranks run through the backend's radix
 *                                          sort (cqlops_sort_rows, cqlops_window_rank), not bitonic passes
 *   qk_filter_spec_kernel, qk_fused_count_spec_kernel
 *                                          0: specialization-constant modules do not exist under NVRTC; the
 *                                          generated scan and fused kernels cover the same programs
 */

#define QK_CUDA_SOURCE_CAP (1u << 20)

internal void
qk_init(void)
{
  QK_State* state = &g_qk_state;
  if (os_handle_match(state->lock, os_handle_zero()))
  {
    state->lock = os_mutex_alloc();
  }
}

/* The backend's kernels are compiled into libcqlcuda.so and found by name: no source is provided. */
internal String8
qk_library_spirv(Arena* arena, String8 name)
{
  (void)arena;
  (void)name;
  return str8_zero();
}

/* FNV-1a over the source, then its length */
internal U64
qk_cuda_key_hash(String8 source)
{
  U64 h = 0xcbf29ce484222325ull;
  for (U64 i = 0; i < source.size; i++)
  {
    h = (h ^ source.str[i]) * 0x100000001b3ull;
  }
  return (h ^ source.size) * 0x100000001b3ull;
}

/* a second hash of another kind: a multiply-rotate over 8-byte words, tail bytes last */
internal U64
qk_cuda_check_hash(String8 source)
{
  U64 h = 0x9e3779b97f4a7c15ull ^ source.size;
  U64 i = 0;
  for (; i + 8 <= source.size; i += 8)
  {
    U64 w = 0;
    MemoryCopy(&w, source.str + i, 8);
    h = (h ^ (w * 0xbf58476d1ce4e5b9ull)) * 0x94d049bb133111ebull;
    h = (h << 31) | (h >> 33);
  }
  for (; i < source.size; i++)
  {
    h = (h ^ source.str[i]) * 0xff51afd7ed558ccdull;
  }
  return h ^ (h >> 29);
}

internal String8
qk_kernel_name_locked(U64 key, U64 check)
{
  QK_State* state = &g_qk_state;
  for (U32 i = 0; i < state->name_count; i++)
  {
    if (state->names[i].key == key && state->names[i].check == check)
    {
      return str8_cstring(state->names[i].text);
    }
  }
  U32 slot = state->name_count;
  if (slot < QK_NAME_CAP)
  {
    state->name_count += 1;
  }
  else
  {
    slot = state->name_next;
    state->name_next = (state->name_next + 1) % QK_NAME_CAP;
  }
  state->names[slot].key = key;
  state->names[slot].check = check;
  snprintf(state->names[slot].text, sizeof(state->names[slot].text), "qk_scan_%016llx%016llx", (unsigned long long)key,
           (unsigned long long)check);
  return str8_cstring(state->names[slot].text);
}

internal String8
qk_kernel_name(U64 key, U64 check)
{
  QK_State* state = &g_qk_state;
  os_mutex_take(state->lock);
  String8 name = qk_kernel_name_locked(key, check);
  os_mutex_drop(state->lock);
  return name;
}

/* NVRTC is linked into the backend; it is usable when a trivial kernel compiles */
internal B32
qk_compiler_available(void)
{
  QK_State* state = &g_qk_state;
  if (!state->library_tried)
  {
    static const char probe[] = "extern \"C\" __global__ void qk_probe(unsigned* p) { if (p) p[0] = 1u; }\n";
    state->library_loaded = cqlcuda_compile_check(probe, sizeof(probe) - 1) ? 1 : 0;
    state->library_tried = 1;
  }
  return state->library_loaded;
}

internal B32
qk_enabled(U64 row_count)
{
  if (settings_u64(str8_lit("QE_PERQUERY_KERNELS"), 1) == 0)
  {
    return 0;
  }
  if (row_count < settings_u64(str8_lit("QE_PERQUERY_MIN_ROWS"), 0))
  {
    return 0;
  }
  return qk_compiler_available();
}

/* QE_BytecodeProgram to the backend's program: the words, constant pool and string pool are the same
   format; each binding keeps its slot and the type it is read as */
internal B32
qk_cuda_program(QE_BytecodeProgram* prog, CqlProgram* out)
{
  MemoryZero(out, sizeof(*out));
  if (prog->word_count > CQLOPS_MAX_WORDS || prog->const_count > CQLOPS_MAX_CONSTS || prog->str_const_pool_size > CQLOPS_MAX_STR_POOL ||
      prog->binding_count > CQLOPS_MAX_BINDINGS)
  {
    return 0;
  }
  MemoryCopy(out->words, prog->words, prog->word_count * sizeof(U32));
  out->word_count = (U32)prog->word_count;
  MemoryCopy(out->consts, prog->consts, prog->const_count * 2 * sizeof(U32));
  out->const_count = (U32)prog->const_count;
  if (prog->str_const_pool_size)
  {
    MemoryCopy(out->str_pool, prog->str_const_pool, prog->str_const_pool_size);
  }
  out->str_pool_size = (U32)prog->str_const_pool_size;
  out->binding_count = prog->binding_count;
  for (U32 i = 0; i < prog->binding_count; i++)
  {
    QE_ColumnBinding* b = &prog->bindings[i];
    out->binding_column[i] = i;
    out->binding_type[i] = b->use_dict_codes ? (U32)CQL_ColumnType_U32 : (U32)b->type;
    out->binding_slot[i] = b->first_slot;
    out->binding_dict[i] = b->use_dict_codes ? 1u : 0u;
  }
  out->next_slot = prog->next_slot;
  out->requires_cpu_scan = prog->requires_cpu_scan ? 1u : 0u;
  out->has_score_output = prog->has_score_output ? (prog->score_is_distance ? 2u : 1u) : 0u;
  return 1;
}

internal B32
qk_scan_source_build(Arena* arena, QE_BytecodeProgram* prog, QK_HybridInfo* hybrid, QK_FusedAgg* fuse, String8* out_source)
{
  if (hybrid)
  {
    hybrid->is_hybrid = 0;
    hybrid->leaf_count = 0;
    hybrid->wide_slot_mask = 0;
  }
  CqlProgram* cp = (CqlProgram*)malloc(sizeof(CqlProgram));
  char* text = (char*)malloc(QK_CUDA_SOURCE_CAP);
  B32 ok = cp && text && qk_cuda_program(prog, cp);
  uint32_t kind = CQLOPS_KERNEL_SCAN;
  CqlFusedAgg f;
  MemoryZero(&f, sizeof(f));
  if (ok && fuse)
  {
    if (fuse->column_count > 4 || fuse->key_count > 3)
    {
      ok = 0;
    }
    else
    {
      kind = fuse->grouped ? CQLOPS_KERNEL_FUSED_GROUP : CQLOPS_KERNEL_FUSED_AGG;
      f.column_count = fuse->column_count;
      f.grouped = fuse->grouped ? 1u : 0u;
      f.key_count = fuse->key_count;
      f.group_count = fuse->group_count;
      for (U32 c = 0; c < fuse->column_count; c++)
      {
        f.slots[c] = fuse->slots[c];
        f.coltypes[c] = fuse->coltypes[c];
      }
      for (U32 k = 0; k < fuse->key_count; k++)
      {
        f.key_slots[k] = fuse->key_slots[k];
        f.key_types[k] = fuse->key_types[k];
        f.key_ranges[k] = fuse->key_ranges[k];
      }
    }
  }
  uint64_t len = 0;
  ok = ok && cqlops_program_source(cp, kind, fuse ? &f : 0, text, QK_CUDA_SOURCE_CAP, &len);
  if (ok)
  {
    U8* copy = push_array_no_zero(arena, U8, len + 1);
    MemoryCopy(copy, text, len + 1);
    *out_source = str8(copy, len);
  }
  free(cp);
  free(text);
  return ok;
}

/* The image kernel_alloc_from_spirv takes under this backend is the CUDA C++ source itself. */
internal String8
qk_spirv_compile(Arena* arena, String8 source)
{
  (void)arena;
  QK_State* state = &g_qk_state;
  state->last_source_bytes = source.size;
  state->last_spirv_bytes = source.size;
  return source;
}

internal GPU_Kernel*
qk_kernel_from_source(Arena* arena, String8 source, String8* out_name)
{
  QK_State* state = &g_qk_state;
  U64 key = qk_cuda_key_hash(source);
  U64 bits = settings_u64(str8_lit("QE_TEST_KEY_BITS"), 0);
  if (bits > 0 && bits < 64)
  {
    key &= (1ull << bits) - 1;
  }
  U64 check = settings_u64(str8_lit("QE_COLLISION_CHECK"), 1) != 0 ? qk_cuda_check_hash(source) : 0;
  U64 memo = key ^ (check * 0x9e3779b97f4a7c15ull);
  os_mutex_take(state->lock);
  for (U32 i = 0; i < state->failed_key_count; i++)
  {
    if (state->failed_keys[i] == memo)
    {
      os_mutex_drop(state->lock);
      return 0;
    }
  }
  String8 name = qk_kernel_name_locked(key, check);
  os_mutex_drop(state->lock);
  GPU_Kernel* kernel = gpu_kernel_alloc_from_spirv(name, str8_zero());
  if (!kernel)
  {
    os_mutex_take(state->lock);
    U64 every = settings_u64(str8_lit("QE_TEST_FAIL_SHADERC"), 0);
    B32 inject = 0;
    if (every)
    {
      state->test_shaderc_count += 1;
      inject = (state->test_shaderc_count % every) == 0;
    }
    os_mutex_drop(state->lock);
    if (!inject)
    {
      kernel = gpu_kernel_alloc_from_spirv(name, qk_spirv_compile(arena, source));
    }
    os_mutex_take(state->lock);
    if (!kernel)
    {
      state->compile_failures += 1;
      if (state->failed_key_count < QK_FAILED_KEY_CAP)
      {
        state->failed_keys[state->failed_key_count++] = memo;
      }
    }
    else
    {
      state->kernels_compiled += 1;
    }
    os_mutex_drop(state->lock);
  }
  if (kernel && out_name)
  {
    *out_name = name;
  }
  return kernel;
}

/* QE_ROUTE_CONJUNCTIONS defers the compile of a conjunction of plain comparisons to its second sighting.
   Here such a conjunction runs on scan_simple (qk_simple_kernel), which compiles nothing, so nothing is
   ever deferred. */
internal U64 qk_routed_deferrals(void) { return g_qk_state.routed_deferrals; }

internal GPU_Kernel*
qk_scan_kernel(Arena* arena, QE_BytecodeProgram* prog, QK_HybridInfo* hybrid, String8* out_name)
{
  if (!qk_compiler_available())
  {
    return 0;
  }
  g_qk_state.kernels_requested += 1;
  String8 source = { 0 };
  if (!qk_scan_source_build(arena, prog, hybrid, 0, &source))
  {
    return 0;
  }
  return qk_kernel_from_source(arena, source, out_name);
}

internal GPU_Kernel*
qk_simple_kernel(Arena* arena, U32* words, String8* out_name)
{
  (void)arena;
  (void)words;
  if (out_name)
  {
    *out_name = str8_lit("scan_simple");
  }
  return gpu_kernel_alloc(str8_lit("scan_simple"));
}

internal GPU_Kernel*
qk_fused_aggregate_kernel(Arena* arena, QE_BytecodeProgram* prog, QK_FusedAgg* fuse, String8* out_name)
{
  if (!qk_compiler_available())
  {
    return 0;
  }
  g_qk_state.kernels_requested += 1;
  String8 source = { 0 };
  if (!qk_scan_source_build(arena, prog, 0, fuse, &source))
  {
    return 0;
  }
  return qk_kernel_from_source(arena, source, out_name);
}

internal GPU_Kernel*
qk_having_kernel(Arena* arena, String8 condition, String8* out_name)
{
  if (!qk_compiler_available() || condition.size == 0 || condition.size > 4096)
  {
    return 0;
  }
  g_qk_state.kernels_requested += 1;
  char* cond = (char*)malloc(condition.size + 1);
  char* text = (char*)malloc(QK_CUDA_SOURCE_CAP);
  uint64_t len = 0;
  B32 ok = cond && text;
  if (ok)
  {
    MemoryCopy(cond, condition.str, condition.size);
    cond[condition.size] = 0;
    ok = cqlops_having_source(cond, 8, text, QK_CUDA_SOURCE_CAP, &len);
  }
  String8 source = { 0 };
  if (ok)
  {
    U8* copy = push_array_no_zero(arena, U8, len + 1);
    MemoryCopy(copy, text, len + 1);
    source = str8(copy, len);
  }
  free(cond);
  free(text);
  return ok ? qk_kernel_from_source(arena, source, out_name) : 0;
}

internal U32
qk_sort_tile(U32 key_count, B32 narrow)
{
  (void)key_count;
  (void)narrow;
  return 4096;
}

internal GPU_Kernel* qk_sort_kernel(Arena* arena, U32 key_count, U32 dir_mask, B32 narrow, String8* out_name)
{
  (void)arena; (void)key_count; (void)dir_mask; (void)narrow; (void)out_name;
  return 0;
}

internal GPU_Kernel* qk_join_build_kernel(Arena* arena, B32 string_key, String8* out_name)
{
  (void)arena; (void)string_key; (void)out_name;
  return 0;
}

internal GPU_Kernel* qk_join_probe_hash_kernel(Arena* arena, B32 string_key, B32 emit_unmatched, String8* out_name)
{
  (void)arena; (void)string_key; (void)emit_unmatched; (void)out_name;
  return 0;
}

internal GPU_Kernel* qk_join_probe_native_kernel(Arena* arena, U64 shader_widths, U32 arg_count, U32 num_exprs, U32 func_codes,
                                                 U32 arg_index_codes, U32 arg_signed_bits, String8* out_name)
{
  (void)arena; (void)shader_widths; (void)arg_count; (void)num_exprs; (void)func_codes; (void)arg_index_codes; (void)arg_signed_bits;
  (void)out_name;
  return 0;
}

internal GPU_Kernel* qk_hash_assign_kernel(Arena* arena, U32 num_group_cols, U32 string_mask, String8* out_name)
{
  (void)arena; (void)num_group_cols; (void)string_mask; (void)out_name;
  return 0;
}

internal GPU_Kernel* qk_member_reduce_kernel(Arena* arena, B32 narrow, U32 num_exprs, U32 func_codes, String8* out_name)
{
  (void)arena; (void)narrow; (void)num_exprs; (void)func_codes; (void)out_name;
  return 0;
}

internal GPU_Kernel* qk_compact_kernel(Arena* arena, String8* out_name)
{
  (void)arena; (void)out_name;
  return 0;
}

internal GPU_Kernel* qk_hash_reduce_kernel(Arena* arena, B32 fixed, U32 num_exprs, U32 func_codes, U32 scales, String8* out_name)
{
  (void)arena; (void)fixed; (void)num_exprs; (void)func_codes; (void)scales; (void)out_name;
  return 0;
}

internal GPU_Kernel* qk_gather_kernel(Arena* arena, U32 mode, String8* out_name)
{
  (void)arena; (void)mode; (void)out_name;
  return 0;
}

internal GPU_Kernel* qk_window_flags_kernel(Arena* arena, U32 key_count, U32 partition_count, B32 narrow, String8* out_name)
{
  (void)arena; (void)key_count; (void)partition_count; (void)narrow; (void)out_name;
  return 0;
}

internal GPU_Kernel* qk_filter_spec_kernel(U32* words, U32 word_count, U32 variant, String8* out_name)
{
  (void)words; (void)word_count; (void)variant; (void)out_name;
  return 0;
}

internal GPU_Kernel* qk_fused_count_spec_kernel(U32 leaf_count, U32* slots, U32* types, U32* ops, String8* out_name)
{
  (void)leaf_count; (void)slots; (void)types; (void)ops; (void)out_name;
  return 0;
}

internal void
qk_last_sizes(U64* out_source_bytes, U64* out_spirv_bytes)
{
  if (out_source_bytes) *out_source_bytes = g_qk_state.last_source_bytes;
  if (out_spirv_bytes) *out_spirv_bytes = g_qk_state.last_spirv_bytes;
}

internal U64 qk_spec_request_count(void) { return g_qk_state.spec_requests; }
internal U64 qk_count_spec_request_count(void) { return g_qk_state.count_spec_requests; }

internal void
qk_stats(U64* out_requested, U64* out_compiled, U64* out_failures, U64* out_compile_microseconds)
{
  QK_State* state = &g_qk_state;
  if (out_requested) *out_requested = state->kernels_requested;
  if (out_compiled) *out_compiled = state->kernels_compiled;
  if (out_failures) *out_failures = state->compile_failures;
  if (out_compile_microseconds) *out_compile_microseconds = state->compile_microseconds;
}
