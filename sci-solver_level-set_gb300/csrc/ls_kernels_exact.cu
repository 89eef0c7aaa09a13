// ls_kernels_exact.cu -- bit-exact build of the step kernels: the same
// source as ls_kernels.cu compiled with -fmad=false, so every float
// operation is an individually rounded IEEE operation in the reference's
// order (the CPU oracle's arithmetic).
#include <cuda_runtime.h>

#include "ls_device.cuh"
#include "ls_solver.h"

#define LS_KERNELS_EXACT 1
namespace lsgb {
namespace exact {
#include "ls_kernels_impl.cuh"
}  // namespace exact
const KernelSet& kernels_exact() { return exact::kernel_table(); }
}  // namespace lsgb
