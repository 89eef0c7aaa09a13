// ls_kernels.cu -- fast build of the step kernels (FMA contraction on).
#include <cuda_runtime.h>

#include "ls_device.cuh"
#include "ls_solver.h"

namespace lsgb {
namespace fast {
#include "ls_kernels_impl.cuh"
}  // namespace fast
const KernelSet& kernels_fast() { return fast::kernel_table(); }
}  // namespace lsgb
