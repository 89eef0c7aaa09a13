// ls_noalloc.cu -- narrowband selection that allocates no device memory.
//
// For callers that cannot call cudaMalloc (or any allocating library
// routine) on the device they run on: a host application that owns every
// device allocation through its own pool, or code running under a fixed
// memory budget, where an allocation inside the call is not allowed (it
// would take memory the caller has already handed out, or fail once the
// budget is spent).  They keep their own device buffers for
// the inputs and outputs; the kernel's scratch (the compact list of
// narrowband patches and the counters) lives in the file-scope device array
// below, sized for at most LS_NOALLOC_MAX_PATCHES patches.
//
// The array exists once per device in every process that loads the library
// and is held until exit.  Its device address is looked up on the first call
// on each device (cudaGetSymbolAddress with that device current); make that
// first call before any stream capture.  Every call shares the array and it
// keeps the previous call's contents: the counters are cleared at the start
// of each call, and calls that overlap on the GPU (different streams, or
// different host threads on the same device) race on it.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/lsgb300.h"

namespace {

constexpr int kMaxPatches = LS_NOALLOC_MAX_PATCHES;
// [0] list length, [2..3] vertex-update count (u64), [4..5] vertices of listed patches (u64)
constexpr int kCounters = 64;
constexpr int kMaxDevices = 64;

// scratch: kCounters ints of counters, then the patch list
static __device__ __align__(256) int g_nb_scratch[kCounters + kMaxPatches];

std::mutex g_mu;
int* g_scratch_ptr[kMaxDevices] = {nullptr};

// Float bits -> unsigned key with the same order as the floats (negative
// values, -0.0 included, rank below +0.0), and back.  For dt >= +0 the key
// order is the bit order the solver's narrowband kernel compares.
__device__ __forceinline__ unsigned order_key(float f) {
  const unsigned b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float order_key_value(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Same selection as the solver's narrowband kernel: a patch is in the
// narrowband when the minimum distance of its owned vertices is at most the
// bandwidth; phi = +-DT * scale (+-DT when DT >= largenum); vertices with
// DT <= bandwidth are counted as vertex updates.  The minimum is taken over
// order keys, so any dt the caller passes (negative values and -0.0 too)
// ranks as the floats do.
__global__ void k_narrowband_noalloc(int nparts, const int* __restrict__ vert_off, const float* __restrict__ dt,
                                     const uint8_t* __restrict__ sign, float bandwidth, float scale,
                                     float largenum, float* __restrict__ phi, int* scratch) {
  __shared__ unsigned long long s_cnt, s_pv;
  if (threadIdx.x == 0) { s_cnt = 0; s_pv = 0; }
  __syncthreads();
  int* list = scratch + kCounters;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned cnt = 0, pv = 0;
  for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < nparts; p += nwarps) {
    const int vs = vert_off[p], ve = vert_off[p + 1];
    unsigned mn = order_key(__int_as_float(0x7f800000));
    for (int v = vs + lane; v < ve; v += 32) {
      const float d = dt[v];
      mn = min(mn, order_key(d));
      cnt += (d <= bandwidth);
      const float mag = (d >= largenum || scale == 1.f) ? d : d * scale;
      phi[v] = sign[v] ? mag : -mag;
    }
    mn = __reduce_min_sync(0xffffffffu, mn);
    if (lane == 0 && order_key_value(mn) <= bandwidth) {
      const int pos = atomicAdd(&scratch[0], 1);
      list[pos] = p;
      pv += ve - vs;
    }
  }
  atomicAdd(&s_cnt, (unsigned long long)cnt);
  if (lane == 0) atomicAdd(&s_pv, (unsigned long long)pv);
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(reinterpret_cast<unsigned long long*>(scratch + 2), s_cnt);
    atomicAdd(reinterpret_cast<unsigned long long*>(scratch + 4), s_pv);
  }
}

// narrowband list (scratch) -> one flag per patch (output, cleared before)
__global__ void k_set_flags(const int* scratch, unsigned char* flags) {
  const int n = scratch[0];
  const int* list = scratch + kCounters;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) flags[list[i]] = 1;
}

}  // namespace

extern "C" ls_status ls_narrowband_noalloc(int nv, int nparts, const int* vert_offsets, const float* dt,
                                           const unsigned char* sign, float bandwidth, float scale,
                                           float largenum, float* phi, unsigned char* nb_flags,
                                           long long* counts, void* stream) {
  if (nparts <= 0 || nv <= 0 || !vert_offsets || !dt || !sign || !phi || !nb_flags || !counts)
    return LS_BAD_INPUT;
  if (nparts > kMaxPatches) return LS_BAD_INPUT;  // beyond the scratch array's capacity
  if (!(scale > 0.f)) return LS_BAD_INPUT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return LS_CUDA_ERROR;
  int* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
      // host code may not take the address of g_nb_scratch directly (that
      // is a host-side stand-in); ask the runtime for the device address
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_nb_scratch) != cudaSuccess || !p) return LS_CUDA_ERROR;
      g_scratch_ptr[dev] = static_cast<int*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(scratch, 0, sizeof(int) * kCounters, st) != cudaSuccess) return LS_CUDA_ERROR;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return LS_CUDA_ERROR;
  k_narrowband_noalloc<<<sms * 8, 256, 0, st>>>(nparts, vert_offsets, dt, sign, bandwidth, scale, largenum, phi,
                                                 scratch);
  if (cudaGetLastError() != cudaSuccess) return LS_CUDA_ERROR;
  if (cudaMemsetAsync(nb_flags, 0, (size_t)nparts, st) != cudaSuccess) return LS_CUDA_ERROR;
  k_set_flags<<<sms * 4, 256, 0, st>>>(scratch, nb_flags);
  if (cudaGetLastError() != cudaSuccess) return LS_CUDA_ERROR;
  // counts: [0] narrowband patches, [1] vertex updates, [2] vertices of the narrowband patches
  int c[6] = {0, 0, 0, 0, 0, 0};
  if (cudaMemcpyAsync(c, scratch, sizeof(c), cudaMemcpyDeviceToHost, st) != cudaSuccess) return LS_CUDA_ERROR;
  if (cudaStreamSynchronize(st) != cudaSuccess) return LS_CUDA_ERROR;
  unsigned long long v1, v2;
  static_assert(sizeof(unsigned long long) == 2 * sizeof(int), "counter layout");
  __builtin_memcpy(&v1, c + 2, sizeof(v1));
  __builtin_memcpy(&v2, c + 4, sizeof(v2));
  counts[0] = c[0];
  counts[1] = (long long)v1;
  counts[2] = (long long)v2;
  return LS_OK;
}
