// Kernel family placeholder: filled in as the hash kernels are built.
#include "cql_internal.cuh"

const CqlKernelDesc cql_kernels_hash[] = {
  { nullptr, nullptr },
};
