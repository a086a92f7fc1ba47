// Kernel family placeholder: filled in as the join kernels are built.
#include "cql_internal.cuh"

const CqlKernelDesc cql_kernels_join[] = {
  { nullptr, nullptr },
};
