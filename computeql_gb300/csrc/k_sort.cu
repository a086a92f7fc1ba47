// Kernel family placeholder: filled in as the sort kernels are built.
#include "cql_internal.cuh"

const CqlKernelDesc cql_kernels_sort[] = {
  { nullptr, nullptr },
};
