/*
 * Host execution of the reference's patch-layout kernels (test
 * infrastructure only, built into oracle/_ref/ by oracle/build_ref.py).
 *
 * The reference builds its patch layout with device kernels launched from
 * meshFIM3d::InitPatches / InitPatches2 / GenerateBlockNeighbors
 * (src/core3d/cuda/meshFIM3d.cu:423-570, kernels in
 * src/core3d/include/meshFIM_kernels.h:410-659) and their 2D twins
 * (src/core2d/cuda/meshFIM2d.cu:447-606, src/core2d/include/
 * meshFIM2d_kernels.h:364-677).  Those translation units are compiled from
 * the reference tree with nvcc, unchanged, with host containers in place of
 * device ones (LSREF_HOST_ONLY).  This file, compiled with the host compiler
 * and linked in place of the CUDA runtime, makes their kernel launches run on
 * the CPU:
 *   - the kernel header is included a second time inside namespace
 *     lsref_host with the CUDA qualifiers defined away, so every kernel body
 *     is also an ordinary host function; blockIdx / threadIdx / blockDim /
 *     gridDim are host variables of that namespace;
 *   - the launch entry points the compiler's launch stubs call
 *     (__cudaPushCallConfiguration, __cudaPopCallConfiguration,
 *     __cudaGetKernel, __cudaLaunchKernel) and the fat-binary registration
 *     hooks are defined here: a launch looks up the host copy of the kernel
 *     by the stub's address and runs it for every block and thread in turn.
 * The layout kernels have no shared memory, barriers or atomics, and every
 * thread writes its own elements, so running the threads one after another
 * gives what any interleaving gives on a GPU.
 *
 * findPartIndicesNegStartKernel reads one element past its input array
 * (array[idx + 1] for idx = size - 1).  Its launch here passes a copy with
 * one element appended (the last value repeated); the value read there only
 * decides a write that the caller overwrites right after the launch
 * (partIndices[size - 1], meshFIM3d.cu:710), so the output does not depend
 * on it.
 *
 * LSREF_DIM selects the 3D (3) or 2D (2) kernel set.
 */
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <utility>
#include <vector>

#include <cutil.h>
#include <cuda_runtime_api.h>

namespace lsref_host {
struct Index3 {
  unsigned x, y, z;
};
Index3 blockIdx, threadIdx, blockDim, gridDim;
char s_array[1];  // the update kernels' dynamic shared memory (never launched here)
using std::max;
using std::min;
}  // namespace lsref_host

#define __global__
#define __device__
#define __host__
#define __shared__
#define __syncthreads() ((void)0)
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

std::vector<int> g_ipermute;  // vert_ipermute as the reference's kernel left it
int g_launches = 0, g_unknown = 0;

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

struct Entry {
  const void* stub;
  void (*run)(void** args);
};

const Entry kTable[] = {
    {(const void*)&LSREF_K(kernel_compute_ele_npart),
     [](void** a) { call_unpacked(&lsref_host::LSREF_K(kernel_compute_ele_npart), a); }},
    {(const void*)&LSREF_K(kernel_fill_ele_label),
     [](void** a) { call_unpacked(&lsref_host::LSREF_K(kernel_fill_ele_label), a); }},
    {(const void*)&LSREF_K(kernel_fill_sequence),
     [](void** a) { call_unpacked(&lsref_host::LSREF_K(kernel_fill_sequence), a); }},
    {(const void*)&LSREF_K(kernel_compute_vert_ipermute), run_vert_ipermute},
    {(const void*)&LSREF_K(kernel_ele_and_vert),
     [](void** a) { call_unpacked(&lsref_host::LSREF_K(kernel_ele_and_vert), a); }},
    {(const void*)&LSREF_K(kernel_compute_local_coords),
     [](void** a) { call_unpacked(&lsref_host::LSREF_K(kernel_compute_local_coords), a); }},
    {(const void*)&LSREF_K(mapAdjacencyToBlockKernel),
     [](void** a) { call_unpacked(&lsref_host::LSREF_K(mapAdjacencyToBlockKernel), a); }},
    {(const void*)&LSREF_K(findPartIndicesNegStartKernel), run_find_part_indices},
};

struct Config {
  dim3 grid, block;
  size_t smem;
  void* stream;
};
Config g_cfg;

}  // namespace

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

cudaError_t __cudaLaunchKernel(cudaKernel_t kernel, dim3 grid, dim3 block, void** args, size_t, cudaStream_t) {
  const void* stub = (const void*)kernel;
  const Entry* e = nullptr;
  for (const Entry& t : kTable)
    if (t.stub == stub) e = &t;
  if (!e) {
    g_unknown++;
    return cudaErrorInvalidDeviceFunction;
  }
  g_launches++;
  lsref_host::gridDim = {grid.x, grid.y, grid.z};
  lsref_host::blockDim = {block.x, block.y, block.z};
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx)
        for (unsigned tz = 0; tz < block.z; ++tz)
          for (unsigned ty = 0; ty < block.y; ++ty)
            for (unsigned tx = 0; tx < block.x; ++tx) {
              lsref_host::blockIdx = {bx, by, bz};
              lsref_host::threadIdx = {tx, ty, tz};
              e->run(args);
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
void __cudaRegisterFunction(void**, const char*, char*, const char*, int, void*, void*, void*, void*, int*) {}
void __cudaRegisterVar(void**, char*, char*, const char*, int, size_t, int, int) {}

// Kernel launches run since the last call, launches of kernels with no host
// copy here, and vert_ipermute as the last permutation kernel left it.
int lsref_host_launches(int* unknown) {
  const int n = g_launches;
  if (unknown) *unknown = g_unknown;
  g_launches = 0;
  g_unknown = 0;
  return n;
}
int lsref_host_ipermute(int* out, int n) {
  if ((int)g_ipermute.size() != n) return -1;
  std::memcpy(out, g_ipermute.data(), sizeof(int) * n);
  return 0;
}

}  // extern "C"
