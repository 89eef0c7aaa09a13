/*
 * Host execution of the reference's kernels (test infrastructure only, built
 * into oracle/_ref/ by oracle/build_ref.py).
 *
 * The reference's time step runs as device kernels launched from host code:
 * the patch layout (meshFIM3d::InitPatches / InitPatches2 /
 * GenerateBlockNeighbors, src/core3d/cuda/meshFIM3d.cu:423-570), the seed
 * search, sign capture, FIM sweeps, checks, reductions and narrowband
 * (redistance3d.cu:10-274 with src/core3d/include/redistance_kernels3d.h)
 * and the advection update (meshFIM3d.cu:83-99, meshFIM_kernels.h:36-408),
 * plus the 2D twins of the layout (meshFIM2d.cu:447-606).  Those translation
 * units are compiled from the reference tree with nvcc, unchanged, with host
 * containers in place of device ones (LSREF_HOST_ONLY).  This file, compiled
 * with the host compiler and linked in place of the CUDA runtime, makes
 * their kernel launches run on the CPU:
 *   - the kernel headers are included a second time inside namespace
 *     lsref_host with the CUDA qualifiers defined away, so every kernel body
 *     is also an ordinary host function; blockIdx / threadIdx / blockDim /
 *     gridDim are host variables of that namespace, __shared__ variables
 *     are function statics (blocks run one after another) and the dynamic
 *     shared-memory array is one buffer of this file (the build makes the
 *     headers' `extern __shared__ char s_array[]` declaration point at it,
 *     the only line it changes);
 *   - every thread of a block is a fiber (ucontext) with its own stack;
 *     __syncthreads() returns to the block scheduler, which resumes the
 *     threads one after another, so a barrier completes when every thread
 *     that has not exited has reached it (exited threads no longer take
 *     part, as on the GPU);
 *   - atomicInc / atomicAdd are plain read-modify-writes (one thread runs at
 *     a time), and sqrt / fabs / fmin / fmax of floats are the float
 *     overloads, as in device code;
 *   - the launch entry points the compiler's launch stubs call
 *     (__cudaPushCallConfiguration, __cudaPopCallConfiguration,
 *     __cudaGetKernel, __cudaLaunchKernel) and the fat-binary registration
 *     hooks are defined here: a launch looks up the host copy of the kernel
 *     by the stub's address and runs it block by block.
 *
 * findPartIndicesNegStartKernel reads one element past its input array
 * (array[idx + 1] for idx = size - 1).  Its launch here passes a copy with
 * one element appended (the last value repeated); the value read there only
 * decides a write that the caller overwrites right after the launch
 * (partIndices[size - 1], meshFIM3d.cu:710), so the output does not depend
 * on it.
 *
 * LSREF_DIM selects the 3D (3: layout, redistance and update kernels) or 2D
 * (2: layout kernels) set.
 */
#include <ucontext.h>

#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include <cutil.h>
#include <cuda_runtime_api.h>

namespace lsref_host {
struct Index3 {
  unsigned x, y, z;
};
Index3 blockIdx, threadIdx, blockDim, gridDim;
alignas(256) char dyn_smem[1 << 20];  // the kernels' dynamic shared memory (one block at a time)
void syncthreads();
inline unsigned atomicInc(unsigned* a, unsigned limit) {
  const unsigned old = *a;
  *a = (old >= limit) ? 0u : old + 1u;
  return old;
}
inline int atomicAdd(int* a, int v) {
  const int old = *a;
  *a += v;
  return old;
}
using std::max;
using std::min;
// float arguments take the float overloads, as CUDA's device math library
// gives them (without these, ::sqrt(double) would widen float expressions)
using std::fabs;
using std::fmax;
using std::fmin;
using std::sqrt;
#if LSREF_DIM == 3
// the label values of redistance3d.h:22-25 (the class itself needs the
// reference's containers, which this file does not include)
#define REDIST3d_H
struct redistance3d {
  enum LabelType { SeedPoint, ActivePoint, AlivePoint, FarPoint };
};
#endif
}  // namespace lsref_host

#define __global__
#define __device__
#define __host__
#define __shared__ static
#define __syncthreads() lsref_host::syncthreads()
// _EPS as meshFIM3d.h (1e-5) and meshFIM2d.h (1e-12) define it; only kernels
// that are not run here read it
#ifndef _EPS
#if LSREF_DIM == 3
#define _EPS 1e-5
#else
#define _EPS 1e-12
#endif
#endif
namespace lsref_host {
#if LSREF_DIM == 3
#include <meshFIM_kernels.h>
#include <redistance_kernels3d.h>
#else
#include <meshFIM2d_kernels.h>
#endif
}  // namespace lsref_host
#undef __global__
#undef __device__
#undef __host__
#undef __shared__
#undef __syncthreads

// The launch stubs of the reference's kernels (the host-side functions the
// compiler generates under each kernel's own name and signature).
#if LSREF_DIM == 3
void kernel_compute_ele_npart3d(int, int*, int*, int*);
void kernel_fill_ele_label3d(int, int*, int*, int*, int*, int*);
void kernel_fill_sequence3d(int, int*);
void kernel_compute_vert_ipermute3d(int, int*, int*);
void kernel_ele_and_vert3d(int, int, int*, int*, int*, int, float*, float*, float*, float*, int*, int*);
void kernel_compute_local_coords3d(int, int, int*, int*, float*, float*, float*, float*);
void mapAdjacencyToBlockKernel3d(int, int*, int*, int*, int*, int*);
void findPartIndicesNegStartKernel3d(int, int*, int*);
void run_reduction3d(int*, int*, int*, int*);
void kernel_update_values(int*, int*, int, int, int, int*, int*, int*, float*, float*, int, int*, int*, int, float*,
                          int*);
void kernel_run_check_neghbor(int*, int*, int, int, int, int*, int*, int*, float*, float*, int, int*, int*, int,
                              float*, int*);
void kernel_seedlabel(int, int, float*, int*, int*, int*, int*, float*, float*, int*);
void kernel_seedlabel_narrowband(int, int, const int*, float*, int*, int*, int*, int*, float*, float*, int*);
void CopyOutBack(int*, int*, float*, float*);
void kernel_reinit_Tsign(int, float*, char*);
void kernel_recover_Tsign_whole(int, float*, char*);
void CopyOutBack_levelset3d(int*, int*, float*, float*);
void kernel_updateT_single_stage3d(float, int*, int, int, int, int*, int*, float*, int, int*, float*, float*, float*,
                                   int, int*, int*, float*);
void kernel_compute_vertT_before_permute3d(int, int*, float*, float*);
#define LSREF_K(name) name##3d
#else
void kernel_compute_ele_npart2d(int, int*, int*, int*);
void kernel_fill_ele_label2d(int, int*, int*, int*, int*, int*);
void kernel_fill_sequence2d(int, int*);
void kernel_compute_vert_ipermute2d(int, int*, int*);
void kernel_ele_and_vert2d(int, int, int*, int*, int*, int, double*, double*, double*, double*, double*, double*,
                           int*, int*);
void kernel_compute_local_coords2d(int, int, int*, int*, double*, double*, double*, double*);
void mapAdjacencyToBlockKernel2d(int, int*, int*, int*, int*, int*);
void findPartIndicesNegStartKernel2d(int, int*, int*);
#define LSREF_K(name) name##2d
#endif

namespace {

template <typename... A, std::size_t... I>
void call_unpacked(void (*f)(A...), void** args, std::index_sequence<I...>) {
  f(*static_cast<A*>(args[I])...);
}
template <typename... A>
void call_unpacked(void (*f)(A...), void** args) {
  call_unpacked(f, args, std::index_sequence_for<A...>{});
}

// stub address -> mangled kernel name, filled while the library loads (a
// function-local static, constructed on first use, whatever the order in
// which the translation units' initialisers run)
std::vector<std::pair<const void*, std::string>>& registered() {
  static std::vector<std::pair<const void*, std::string>> r;
  return r;
}
std::vector<int> g_ipermute;  // vert_ipermute as the reference's kernel left it
int g_launches = 0, g_failed = 0;

void run_find_part_indices(void** args) {
  // input padded by one element (see the file comment)
  const int size = *static_cast<int*>(args[0]);
  const int* array = *static_cast<int**>(args[1]);
  std::vector<int> padded(array, array + size);
  padded.push_back(size > 0 ? array[size - 1] : 0);
  int* p = padded.data();
  void* a2[3] = {args[0], &p, args[2]};
  call_unpacked(&lsref_host::LSREF_K(findPartIndicesNegStartKernel), a2);
}

void run_vert_ipermute(void** args) {
  call_unpacked(&lsref_host::LSREF_K(kernel_compute_vert_ipermute), args);
  const int nn = *static_cast<int*>(args[0]);
  const int* ip = *static_cast<int**>(args[2]);
  g_ipermute.assign(ip, ip + nn);
}

// A kernel's host copy, found by the address of its launch stub or, for
// the template kernels (whose stubs have internal linkage), by the mangled
// name the stub registers.
struct Entry {
  const void* stub;
  const char* name;
  void (*run)(void** args);
};

#define LSREF_ENTRY(name) \
  { (const void*)&name, nullptr, [](void** a) { call_unpacked(&lsref_host::name, a); } }
#define LSREF_NAMED(mangled, name) \
  { nullptr, mangled, [](void** a) { call_unpacked(&lsref_host::name, a); } }

const Entry kTable[] = {
    LSREF_ENTRY(LSREF_K(kernel_compute_ele_npart)),
    LSREF_ENTRY(LSREF_K(kernel_fill_ele_label)),
    LSREF_ENTRY(LSREF_K(kernel_fill_sequence)),
    {(const void*)&LSREF_K(kernel_compute_vert_ipermute), nullptr, run_vert_ipermute},
    LSREF_ENTRY(LSREF_K(kernel_ele_and_vert)),
    LSREF_ENTRY(LSREF_K(kernel_compute_local_coords)),
    LSREF_ENTRY(LSREF_K(mapAdjacencyToBlockKernel)),
    {(const void*)&LSREF_K(findPartIndicesNegStartKernel), nullptr, run_find_part_indices},
#if LSREF_DIM == 3
    LSREF_NAMED("_Z29kernel_compute_new_narrowbandILi8EEvPiPfS0_f", kernel_compute_new_narrowband<8>),
    LSREF_NAMED("_Z29kernel_compute_new_narrowbandILi16EEvPiPfS0_f", kernel_compute_new_narrowband<16>),
    LSREF_NAMED("_Z29kernel_compute_new_narrowbandILi32EEvPiPfS0_f", kernel_compute_new_narrowband<32>),
    LSREF_NAMED("_Z29kernel_compute_new_narrowbandILi64EEvPiPfS0_f", kernel_compute_new_narrowband<64>),
    LSREF_NAMED("_Z29kernel_compute_new_narrowbandILi128EEvPiPfS0_f", kernel_compute_new_narrowband<128>),
    LSREF_NAMED("_Z29kernel_compute_new_narrowbandILi256EEvPiPfS0_f", kernel_compute_new_narrowband<256>),
    LSREF_NAMED("_Z23run_reduction_bandwidthILi32EEvPiS0_S0_PfS1_S0_", run_reduction_bandwidth<32>),
    LSREF_NAMED("_Z23run_reduction_bandwidthILi64EEvPiS0_S0_PfS1_S0_", run_reduction_bandwidth<64>),
    LSREF_NAMED("_Z23run_reduction_bandwidthILi128EEvPiS0_S0_PfS1_S0_", run_reduction_bandwidth<128>),
    LSREF_NAMED("_Z23run_reduction_bandwidthILi256EEvPiS0_S0_PfS1_S0_", run_reduction_bandwidth<256>),
    LSREF_ENTRY(run_reduction3d),
    LSREF_ENTRY(kernel_update_values),
    LSREF_ENTRY(kernel_run_check_neghbor),
    LSREF_ENTRY(kernel_seedlabel),
    LSREF_ENTRY(kernel_seedlabel_narrowband),
    LSREF_ENTRY(CopyOutBack),
    LSREF_ENTRY(kernel_reinit_Tsign),
    LSREF_ENTRY(kernel_recover_Tsign_whole),
    LSREF_ENTRY(CopyOutBack_levelset3d),
    LSREF_ENTRY(kernel_updateT_single_stage3d),
    LSREF_ENTRY(kernel_compute_vertT_before_permute3d),
#endif
};

struct Config {
  dim3 grid, block;
  size_t smem;
  void* stream;
};
Config g_cfg;

// Block scheduler: one fiber per thread.
constexpr size_t kStack = 128 * 1024;
struct Fiber {
  ucontext_t ctx;
  bool done;
};
ucontext_t g_sched;
std::vector<Fiber> g_fib;
std::vector<char> g_stacks;
unsigned g_cur = 0;
const Entry* g_entry = nullptr;
void** g_args = nullptr;

void fiber_main() {
  g_entry->run(g_args);
  g_fib[g_cur].done = true;  // returns to the scheduler through uc_link
}

bool run_block(unsigned nthreads, const dim3& block) {
  if (g_fib.size() < nthreads) g_fib.resize(nthreads);
  if (g_stacks.size() < nthreads * kStack) g_stacks.resize(nthreads * kStack);
  for (unsigned t = 0; t < nthreads; ++t) {
    Fiber& f = g_fib[t];
    f.done = false;
    if (getcontext(&f.ctx) != 0) return false;
    f.ctx.uc_stack.ss_sp = g_stacks.data() + (size_t)t * kStack;
    f.ctx.uc_stack.ss_size = kStack;
    f.ctx.uc_link = &g_sched;
    makecontext(&f.ctx, fiber_main, 0);
  }
  unsigned live = nthreads;
  while (live > 0) {
    for (unsigned t = 0; t < nthreads; ++t) {
      if (g_fib[t].done) continue;
      g_cur = t;
      lsref_host::threadIdx = {t % block.x, (t / block.x) % block.y, t / (block.x * block.y)};
      if (swapcontext(&g_sched, &g_fib[t].ctx) != 0) return false;
      if (g_fib[t].done) live--;
    }
  }
  return true;
}

}  // namespace

void lsref_host::syncthreads() { swapcontext(&g_fib[g_cur].ctx, &g_sched); }

extern "C" {

// Launch configuration and launch entry points of the compiler's stubs.
unsigned __cudaPushCallConfiguration(dim3 gridDim, dim3 blockDim, size_t sharedMem, void* stream) {
  g_cfg = Config{gridDim, blockDim, sharedMem, stream};
  return 0;
}

cudaError_t __cudaPopCallConfiguration(dim3* gridDim, dim3* blockDim, size_t* sharedMem, void* stream) {
  *gridDim = g_cfg.grid;
  *blockDim = g_cfg.block;
  *sharedMem = g_cfg.smem;
  *static_cast<void**>(stream) = g_cfg.stream;
  return cudaSuccess;
}

cudaError_t __cudaGetKernel(cudaKernel_t* kernel, const void* stub) {
  *kernel = (cudaKernel_t)const_cast<void*>(stub);
  return cudaSuccess;
}

cudaError_t __cudaLaunchKernel(cudaKernel_t kernel, dim3 grid, dim3 block, void** args, size_t smem, cudaStream_t) {
  const void* stub = (const void*)kernel;
  const Entry* e = nullptr;
  for (const Entry& t : kTable)
    if (t.stub && t.stub == stub) e = &t;
  if (!e)
    for (const auto& r : registered())
      if (r.first == stub)
        for (const Entry& t : kTable)
          if (t.name && r.second == t.name) e = &t;
  if (!e || smem > sizeof(lsref_host::dyn_smem)) {
    g_failed++;
    return cudaErrorInvalidDeviceFunction;
  }
  g_launches++;
  g_entry = e;
  g_args = args;
  lsref_host::gridDim = {grid.x, grid.y, grid.z};
  lsref_host::blockDim = {block.x, block.y, block.z};
  const unsigned nthreads = block.x * block.y * block.z;
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        lsref_host::blockIdx = {bx, by, bz};
        if (!run_block(nthreads, block)) {
          g_failed++;
          return cudaErrorLaunchFailure;
        }
      }
  return cudaSuccess;
}

cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }

// Fat-binary registration hooks (the device code is never loaded).
void** __cudaRegisterFatBinary(void*) {
  static void* handle = nullptr;
  return &handle;
}
void __cudaRegisterFatBinaryEnd(void**) {}
void __cudaUnregisterFatBinary(void**) {}
void __cudaRegisterFunction(void**, const char* hostFun, char*, const char* deviceName, int, void*, void*, void*,
                            void*, int*) {
  registered().emplace_back((const void*)hostFun, std::string(deviceName));
}
void __cudaRegisterVar(void**, char*, char*, const char*, int, size_t, int, int) {}

// Kernel launches run since the last call, launches that failed (no host
// copy here, or more dynamic shared memory than the buffer), and
// vert_ipermute as the last permutation kernel left it.
int lsref_host_launches(int* failed) {
  const int n = g_launches;
  if (failed) *failed = g_failed;
  g_launches = 0;
  g_failed = 0;
  return n;
}
int lsref_host_ipermute(int* out, int n) {
  if ((int)g_ipermute.size() != n) return -1;
  std::memcpy(out, g_ipermute.data(), sizeof(int) * n);
  return 0;
}

}  // extern "C"
