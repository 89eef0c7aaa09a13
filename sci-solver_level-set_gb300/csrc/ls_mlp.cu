// ls_mlp.cu -- the learned warm start: a 128-128-128-128-1 ReLU MLP on the
// 5th-generation tensor cores (tcgen05.mma, BF16 operands in shared memory,
// FP32 accumulators in tensor memory), with forward, backward and Adam
// kernels for training on the GPU and a feature kernel that builds the
// network input of a vertex from its 1-ring.
//
// Network (per sample, all layers 128 wide):
//   a0 = bf16(x)                                  x: 32 padded 1-ring slots x
//                                                 (dx, dy, dz, phi) / h
//   z_l = a_l W_l^T (fp32 accumulate) + b_l,      l = 1, 2, 3, W_l [out][in] bf16
//   a_l = bf16(relu(z_l))
//   y   = sum_j a_3[j] w4[j] + b4                 (fp32)
// Loss: 1/(2n) sum (y - t)^2.  Backward in the same precisions:
//   dy = (y - t)/n;  g_w4 = sum dy a_3;  g_b4 = sum dy
//   d_3 = bf16(dy w4 * [a_3 > 0])
//   g_W_l = d_l^T a_{l-1} (fp32 accumulate);  g_b_l = sum_samples d_l
//   d_{l-1} = bf16((d_l W_l) * [a_{l-1} > 0])
//
// One CTA of 128 threads handles a tile of 128 samples.  Operand tiles use
// the no-swizzle K-major core-matrix layout of the tensor core: element
// (row r, k) of a 128 x 128 BF16 tile sits at byte
//   (r / 8) * 2048 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// i.e. 8 x 16-byte core matrices, 128 bytes apart along K (leading byte
// offset) and 2048 bytes apart along M/N (stride byte offset).  One MMA
// (M = N = 128, K = 16) covers two core matrices along K; the K loop
// advances both descriptors by 256 bytes.  The accumulator (M = 128) keeps
// row r in tensor-memory lane r, column n in column n; warp w of the CTA
// reads lanes 32w..32w+31 with tcgen05.ld.
//
// Every wait on an mbarrier is bounded (about one second of clock cycles);
// on expiry the kernel records the error, waits (bounded) for its MMAs,
// frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "ls_mlp.h"

namespace lsgb {
namespace mlp {

namespace {

constexpr int F = 128;        // features = hidden width
constexpr int TILE = 128;     // samples per CTA
constexpr int TILE_BYTES = TILE * F * 2;   // one BF16 operand tile (32 KB)
constexpr uint32_t LBO = 128, SBO = 2048;  // core-matrix strides (bytes)
// kind::f16 instruction descriptor: D fp32 (bits 4-5 = 1), A bf16 (bits
// 7-9 = 1), B bf16 (bits 10-12 = 1), A and B K-major, N >> 3 at bits 17-22,
// M >> 4 at bits 24-28
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(F >> 3) << 17) |
                           ((uint32_t)(TILE >> 4) << 24);
constexpr long long WAIT_CYCLES = 2000000000LL;  // ~1 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint32_t tile_off(int r, int k) {
  return (uint32_t)((r >> 3) * SBO + (k >> 3) * LBO + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor, no swizzle (layout type 0), version 1
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((LBO >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((SBO >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, int accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(IDESC), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// bounded wait for the phase with the given parity to complete
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok = 0;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > WAIT_CYCLES) return false;
  }
}

// 32 consecutive accumulator columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// row r of a [rows][128] BF16 global matrix -> tile row r (16-byte chunks)
__device__ __forceinline__ void load_row(uint8_t* tile, int r, const __nv_bfloat16* src) {
  const uint4* s = reinterpret_cast<const uint4*>(src);
#pragma unroll 4
  for (int j = 0; j < F / 8; ++j) *reinterpret_cast<uint4*>(tile + tile_off(r, j * 8)) = __ldg(s + j);
}

__device__ __forceinline__ void zero_row(uint8_t* tile, int r) {
#pragma unroll 4
  for (int j = 0; j < F / 8; ++j) *reinterpret_cast<uint4*>(tile + tile_off(r, j * 8)) = make_uint4(0, 0, 0, 0);
}

// 8 floats -> 8 BF16 (round to nearest even) in one 16-byte chunk
__device__ __forceinline__ uint4 pack8(const float* v) {
  uint4 o;
  __nv_bfloat162 p0 = __floats2bfloat162_rn(v[0], v[1]);
  __nv_bfloat162 p1 = __floats2bfloat162_rn(v[2], v[3]);
  __nv_bfloat162 p2 = __floats2bfloat162_rn(v[4], v[5]);
  __nv_bfloat162 p3 = __floats2bfloat162_rn(v[6], v[7]);
  o.x = *reinterpret_cast<uint32_t*>(&p0);
  o.y = *reinterpret_cast<uint32_t*>(&p1);
  o.z = *reinterpret_cast<uint32_t*>(&p2);
  o.w = *reinterpret_cast<uint32_t*>(&p3);
  return o;
}

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Issue the 8 K-steps of one 128 x 128 x 128 product (thread 0 only).
__device__ __forceinline__ void mma_tile(uint32_t tmem_d, const uint8_t* a, const uint8_t* b) {
  const uint32_t sa = smem_u32(a), sb = smem_u32(b);
#pragma unroll
  for (int ks = 0; ks < F / 16; ++ks) mma(tmem_d, make_desc(sa + ks * 2 * LBO), make_desc(sb + ks * 2 * LBO), ks > 0);
}

struct Smem {
  uint64_t bar;
  uint32_t tmem;
  int fail;
};

}  // namespace

// ---------------------------------------------------------------------------
// Forward.  X [n][128] BF16; W [3][128][128] BF16 ([out][in]); b [3][128],
// w4 [128], b4 [1] fp32; y [n]; A (optional) [3][n][128] BF16 activations
// a_1..a_3 for the backward pass.  n_dev (optional) overrides n from device
// memory (graph replays with a device-side sample count).
__global__ void __launch_bounds__(128, 1)
    k_mlp_fwd(const __nv_bfloat16* __restrict__ X, int n, const int* n_dev, const __nv_bfloat16* __restrict__ W,
              const float* __restrict__ b, const float* __restrict__ w4, const float* __restrict__ b4,
              float* __restrict__ y, __nv_bfloat16* __restrict__ A, int* err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* act = base;                       // activation tile (A operand)
  uint8_t* wt = base + TILE_BYTES;           // 3 weight tiles (B operands)
  Smem* sm = reinterpret_cast<Smem*>(base + 4 * TILE_BYTES);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (n_dev) n = *n_dev;
  const int s0 = blockIdx.x * TILE;
  if (s0 >= n) return;  // whole CTA exits before any tensor-core work
  if (tid == 0) {
    mbar_init(&sm->bar, 1);
    sm->fail = 0;
  }
  __syncwarp();
  if (warp == 0) tmem_alloc(&sm->tmem, 128);
  // operands: sample row tid, weight row tid of each layer
  const int s = s0 + tid;
  if (s < n) load_row(act, tid, X + (size_t)s * F);
  else zero_row(act, tid);
  for (int l = 0; l < 3; ++l) load_row(wt + l * TILE_BYTES, tid, W + ((size_t)l * F + tid) * F);
  fence_async_smem();
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = sm->tmem;
  uint32_t phase = 0;
  float out = 0.f;
  bool ok = true;
  for (int l = 0; l < 3 && ok; ++l) {
    if (tid == 0) {
      mma_tile(tmem, act, wt + l * TILE_BYTES);
      mma_commit(&sm->bar);
    }
    ok = __syncthreads_and(mbar_wait(&sm->bar, phase)) != 0;
    phase ^= 1;
    if (!ok) break;
    fence_after();
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    const int r = warp * 32 + lane;  // sample row of this thread
    for (int c = 0; c < F / 32; ++c) {
      float v[32];
      tmem_ld32(trow + c * 32, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) v[j] = bf16r(fmaxf(v[j] + __ldg(b + l * F + c * 32 + j), 0.f));
      if (l < 2) {
#pragma unroll
        for (int q = 0; q < 4; ++q) *reinterpret_cast<uint4*>(act + tile_off(r, c * 32 + q * 8)) = pack8(v + q * 8);
      } else {
#pragma unroll
        for (int j = 0; j < 32; ++j) out += v[j] * __ldg(w4 + c * 32 + j);
      }
      if (A && s0 + r < n) {
        uint4* dst = reinterpret_cast<uint4*>(A + ((size_t)l * n + s0 + r) * F + c * 32);
#pragma unroll
        for (int q = 0; q < 4; ++q) dst[q] = pack8(v + q * 8);
      }
    }
    fence_before();
    fence_async_smem();
    __syncthreads();
    fence_after();
  }
  if (ok) {
    const int r = warp * 32 + lane;
    if (s0 + r < n) y[s0 + r] = out + __ldg(b4);
  } else {
    sm->fail = 1;
    if (err) atomicExch(err, 1);
    // drain: wait (bounded) for the MMAs of this phase before freeing TMEM
    mbar_wait(&sm->bar, phase ^ 1);
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0) tmem_dealloc(tmem, 128);
}

// ---------------------------------------------------------------------------
// Backward: gradients accumulated (atomics) into G = [gW (3x128x128) | gb
// (3x128) | gw4 (128) | gb4 (1) | loss (1)], all fp32.  WT [3][in][out]
// BF16 (transposed weights), A the forward activations, t targets.
__global__ void __launch_bounds__(128, 1)
    k_mlp_bwd(const __nv_bfloat16* __restrict__ X, int n, const __nv_bfloat16* __restrict__ WT,
              const float* __restrict__ w4, const __nv_bfloat16* __restrict__ A, const float* __restrict__ y,
              const float* __restrict__ t, float inv_n, float* __restrict__ G, int* err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* dT = base;                   // A operand of gW: d^T  (rows = out, K = samples)
  uint8_t* aT = base + TILE_BYTES;      // B operand of gW: a^T  (rows = in,  K = samples)
  uint8_t* dN = base + 2 * TILE_BYTES;  // A operand of dH: d    (rows = samples, K = out)
  uint8_t* wN = base + 3 * TILE_BYTES;  // B operand of dH: W^T  (rows = in, K = out)
  float* s_gb = reinterpret_cast<float*>(base + 4 * TILE_BYTES);  // [128] bias gradient of the layer
  Smem* sm = reinterpret_cast<Smem*>(base + 4 * TILE_BYTES + F * sizeof(float));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int s0 = blockIdx.x * TILE;
  if (s0 >= n) return;
  if (tid == 0) {
    mbar_init(&sm->bar, 1);
    sm->fail = 0;
  }
  __syncwarp();
  if (warp == 0) tmem_alloc(&sm->tmem, 256);
  float* gW = G;
  float* gb = G + 3 * F * F;
  float* gw4 = gb + 3 * F;
  float* gb4 = gw4 + F;
  float* gloss = gb4 + 1;
  const int r = tid;  // sample row of this thread in the operand phase
  const int s = s0 + r;
  const bool valid = s < n;
  // output layer
  float dy = 0.f;
  if (valid) {
    const float e = y[s] - t[s];
    dy = e * inv_n;
    atomicAdd(gloss, 0.5f * e * e * inv_n);
  }
  {
    float sum = dy;
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) atomicAdd(gb4, sum);
  }
  // d_3 = bf16(dy w4 [a_3 > 0]); gw4 = sum dy a_3
  s_gb[tid] = 0.f;
  __syncthreads();
  {
    const __nv_bfloat16* a3 = A + ((size_t)2 * n + (valid ? s : s0)) * F;
    for (int c = 0; c < F; c += 8) {
      float av[8], dv[8];
      if (valid) {
        const uint4 raw = __ldg(reinterpret_cast<const uint4*>(a3 + c));
        const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&raw);
#pragma unroll
        for (int j = 0; j < 8; ++j) av[j] = __bfloat162float(hb[j]);
      } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) av[j] = 0.f;
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        dv[j] = bf16r(av[j] > 0.f ? dy * __ldg(w4 + c + j) : 0.f);
        atomicAdd(&s_gb[c + j], dv[j]);
      }
      *reinterpret_cast<uint4*>(dN + tile_off(r, c)) = pack8(dv);
#pragma unroll
      for (int j = 0; j < 8; ++j) *reinterpret_cast<__nv_bfloat16*>(dT + tile_off(c + j, r)) = __float2bfloat16_rn(dv[j]);
    }
  }
  // gw4[j] = sum_r dy_r a3[r][j]: warp-reduce per column through shuffles
  {
    const __nv_bfloat16* a3 = A + ((size_t)2 * n + (valid ? s : s0)) * F;
    for (int c = 0; c < F; ++c) {
      float v = valid ? dy * __bfloat162float(a3[c]) : 0.f;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) atomicAdd(gw4 + c, v);
    }
  }
  __syncthreads();
  atomicAdd(gb + 2 * F + tid, s_gb[tid]);
  uint32_t phase = 0;
  bool ok = true;
  for (int l = 2; l >= 0 && ok; --l) {
    // B operand of gW_l: a_{l-1}^T (a_0 = X)
    {
      const __nv_bfloat16* src = l == 0 ? (X + (size_t)(valid ? s : s0) * F)
                                        : (A + ((size_t)(l - 1) * n + (valid ? s : s0)) * F);
      for (int c = 0; c < F; c += 8) {
        uint4 raw = valid ? __ldg(reinterpret_cast<const uint4*>(src + c)) : make_uint4(0, 0, 0, 0);
        const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&raw);
#pragma unroll
        for (int j = 0; j < 8; ++j) *reinterpret_cast<__nv_bfloat16*>(aT + tile_off(c + j, r)) = hb[j];
      }
    }
    // B operand of dH_{l-1} = d_l W_l: rows of W_l^T
    if (l > 0) load_row(wN, r, WT + ((size_t)l * F + r) * F);
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tm = sm->tmem;
    if (tid == 0) {
      mma_tile(tm, dT, aT);                       // gW_l  -> columns [0, 128)
      if (l > 0) mma_tile(tm + 128, dN, wN);      // dH    -> columns [128, 256)
      mma_commit(&sm->bar);
    }
    ok = __syncthreads_and(mbar_wait(&sm->bar, phase)) != 0;
    phase ^= 1;
    if (!ok) break;
    fence_after();
    const int rr = warp * 32 + lane;  // accumulator row of this thread
    const uint32_t trow = tm + ((uint32_t)(warp * 32) << 16);
    // gW_l row rr (output feature rr)
    for (int c = 0; c < F / 32; ++c) {
      float v[32];
      tmem_ld32(trow + c * 32, v);
      float4* dst = reinterpret_cast<float4*>(gW + ((size_t)l * F + rr) * F + c * 32);
#pragma unroll
      for (int q = 0; q < 8; ++q) atomicAdd(dst + q, make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]));
    }
    if (l > 0) {
      // d_{l-1} for sample rr = bf16(dH * [a_{l-1} > 0])
      s_gb[tid] = 0.f;
      fence_before();
      __syncthreads();
      fence_after();
      const int sr = s0 + rr;
      const bool vr = sr < n;
      const __nv_bfloat16* ap = A + ((size_t)(l - 1) * n + (vr ? sr : s0)) * F;
      for (int c = 0; c < F / 32; ++c) {
        float v[32];
        tmem_ld32(trow + 128 + c * 32, v);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const float a = vr ? __bfloat162float(ap[c * 32 + j]) : 0.f;
          v[j] = bf16r(a > 0.f ? v[j] : 0.f);
          atomicAdd(&s_gb[c * 32 + j], v[j]);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) *reinterpret_cast<uint4*>(dN + tile_off(rr, c * 32 + q * 8)) = pack8(v + q * 8);
#pragma unroll
        for (int j = 0; j < 32; ++j)
          *reinterpret_cast<__nv_bfloat16*>(dT + tile_off(c * 32 + j, rr)) = __float2bfloat16_rn(v[j]);
      }
      fence_before();
      __syncthreads();
      fence_after();
      atomicAdd(gb + (l - 1) * F + tid, s_gb[tid]);
    }
    fence_before();
    __syncthreads();
    fence_after();
  }
  if (!ok) {
    sm->fail = 1;
    if (err) atomicExch(err, 1);
    mbar_wait(&sm->bar, phase ^ 1);
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0) tmem_dealloc(sm->tmem, 256);
}

// ---------------------------------------------------------------------------
// Adam on the fp32 master parameters P = [W (3x128x128) | b (3x128) | w4 |
// b4]; refreshes the BF16 copies W and W^T.
__global__ void k_adam(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M1,
                       float* __restrict__ M2, int np, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16* __restrict__ Wb, __nv_bfloat16* __restrict__ WTb) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const float g = G[i];
    const float m = b1 * M1[i] + (1.f - b1) * g;
    const float v = b2 * M2[i] + (1.f - b2) * g * g;
    M1[i] = m;
    M2[i] = v;
    const float p = P[i] - lr * (m * c1) / (sqrtf(v * c2) + eps);
    P[i] = p;
    if (i < 3 * F * F) {
      const int l = i / (F * F), o = (i / F) % F, in = i % F;
      Wb[i] = __float2bfloat16_rn(p);
      WTb[(size_t)l * F * F + (size_t)in * F + o] = __float2bfloat16_rn(p);
    }
  }
}

__global__ void k_pack_weights(const float* __restrict__ P, __nv_bfloat16* __restrict__ Wb,
                               __nv_bfloat16* __restrict__ WTb) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * F * F; i += gridDim.x * blockDim.x) {
    const int l = i / (F * F), o = (i / F) % F, in = i % F;
    Wb[i] = __float2bfloat16_rn(P[i]);
    WTb[(size_t)l * F * F + (size_t)in * F + o] = __float2bfloat16_rn(P[i]);
  }
}

// ---------------------------------------------------------------------------
// Features of the vertices in vlist (product vertex ids): slot 0 = the vertex
// itself (0, 0, 0, phi / h), slots 1..31 = its first 31 1-ring neighbours
// (ascending id) as (dx, dy, dz, phi) / h, zeros beyond the ring.
__global__ void k_features(int nlist, const int* __restrict__ vlist, const int* __restrict__ nlist_dev,
                           const int* __restrict__ adj_off, const int* __restrict__ adj, const float* __restrict__ xyz,
                           int nv, const float* __restrict__ phi, float inv_h, __nv_bfloat16* __restrict__ Xo) {
  if (nlist_dev) nlist = *nlist_dev;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nlist; i += gridDim.x * blockDim.x) {
    const int v = vlist[i];
    const float x0 = xyz[v], y0 = xyz[nv + v], z0 = xyz[2 * (size_t)nv + v];
    const int a = adj_off[v], e = adj_off[v + 1];
    __nv_bfloat16* dst = Xo + (size_t)i * F;
    for (int slot = 0; slot < 32; ++slot) {
      float f[4] = {0.f, 0.f, 0.f, 0.f};
      if (slot == 0) {
        f[3] = phi[v] * inv_h;
      } else if (a + slot - 1 < e) {
        const int u = adj[a + slot - 1];
        f[0] = (xyz[u] - x0) * inv_h;
        f[1] = (xyz[nv + u] - y0) * inv_h;
        f[2] = (xyz[2 * (size_t)nv + u] - z0) * inv_h;
        f[3] = phi[u] * inv_h;
      }
      __nv_bfloat162 p0 = __floats2bfloat162_rn(f[0], f[1]);
      __nv_bfloat162 p1 = __floats2bfloat162_rn(f[2], f[3]);
      uint2 o;
      o.x = *reinterpret_cast<uint32_t*>(&p0);
      o.y = *reinterpret_cast<uint32_t*>(&p1);
      *reinterpret_cast<uint2*>(dst + slot * 4) = o;
    }
  }
}

// Training pairs: rows i < *n of X / t with a finite target are appended to
// the pair buffer (capacity cap; overflow is counted, not written).
__global__ void k_append_pairs(const __nv_bfloat16* __restrict__ X, const float* __restrict__ t, const int* n_dev,
                               __nv_bfloat16* __restrict__ PX, float* __restrict__ PT,
                               unsigned long long* count, long long cap) {
  const int n = *n_dev;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float v = t[i];
    if (!isfinite(v)) continue;
    const unsigned long long pos = atomicAdd(count, 1ull);
    if ((long long)pos >= cap) continue;
    const uint4* src = reinterpret_cast<const uint4*>(X + (size_t)i * F);
    uint4* dst = reinterpret_cast<uint4*>(PX + (size_t)pos * F);
#pragma unroll 4
    for (int j = 0; j < F / 8; ++j) dst[j] = src[j];
    PT[pos] = v;
  }
}

// rows perm[i] of (X, t) -> row i of (Xo, to)
__global__ void k_gather_pairs(const __nv_bfloat16* __restrict__ X, const float* __restrict__ t,
                               const int* __restrict__ perm, long long n, __nv_bfloat16* __restrict__ Xo,
                               float* __restrict__ to) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long j = perm[i];
    const uint4* src = reinterpret_cast<const uint4*>(X + (size_t)j * F);
    uint4* dst = reinterpret_cast<uint4*>(Xo + (size_t)i * F);
#pragma unroll 4
    for (int q = 0; q < F / 8; ++q) dst[q] = src[q];
    to[i] = t[j];
  }
}

// ---------------------------------------------------------------------------
// Host side.

namespace {
constexpr int NP = 3 * F * F + 3 * F + F + 1;  // master parameters
constexpr int NG = NP + 1;                      // gradients + loss
size_t fwd_smem() { return 4 * (size_t)TILE_BYTES + 1024 + 64; }
size_t bwd_smem() { return 4 * (size_t)TILE_BYTES + F * sizeof(float) + 1024 + 64; }
}  // namespace

#define MLP_TRY(expr, what)                                                     \
  do {                                                                          \
    cudaError_t _e = (expr);                                                    \
    if (_e != cudaSuccess) return std::string(what) + ": " + cudaGetErrorString(_e); \
  } while (0)

Net::~Net() {
  for (void* p : allocs_) cudaFree(p);
  if (PX_) cudaFree(PX_);
  if (PT_) cudaFree(PT_);
  if (pair_count_) cudaFree(pair_count_);
  if (stream_) cudaStreamDestroy(stream_);
}

std::string Net::init(unsigned long long seed) {
  MLP_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
  auto alloc = [&](void** p, size_t bytes) -> cudaError_t {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) allocs_.push_back(*p);
    return e;
  };
  MLP_TRY(alloc((void**)&P_, sizeof(float) * NP), "alloc");
  MLP_TRY(alloc((void**)&G_, sizeof(float) * NG), "alloc");
  MLP_TRY(alloc((void**)&M1_, sizeof(float) * NP), "alloc");
  MLP_TRY(alloc((void**)&M2_, sizeof(float) * NP), "alloc");
  MLP_TRY(alloc((void**)&Wb_, sizeof(__nv_bfloat16) * 3 * F * F), "alloc");
  MLP_TRY(alloc((void**)&WTb_, sizeof(__nv_bfloat16) * 3 * F * F), "alloc");
  MLP_TRY(alloc((void**)&err_, sizeof(int)), "alloc");
  MLP_TRY(cudaMemsetAsync(M1_, 0, sizeof(float) * NP, stream_), "memset");
  MLP_TRY(cudaMemsetAsync(M2_, 0, sizeof(float) * NP, stream_), "memset");
  MLP_TRY(cudaMemsetAsync(err_, 0, sizeof(int), stream_), "memset");
  MLP_TRY(cudaFuncSetAttribute(k_mlp_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwd_smem()), "attr");
  MLP_TRY(cudaFuncSetAttribute(k_mlp_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bwd_smem()), "attr");
  // He-uniform initialisation of the weights, zero biases
  std::mt19937_64 rng(seed);
  std::vector<float> p(NP, 0.f);
  const float lim = std::sqrt(6.f / F);
  std::uniform_real_distribution<float> U(-lim, lim);
  for (int i = 0; i < 3 * F * F; ++i) p[i] = U(rng);
  std::uniform_real_distribution<float> U4(-std::sqrt(3.f / F), std::sqrt(3.f / F));
  for (int i = 0; i < F; ++i) p[3 * F * F + 3 * F + i] = U4(rng);
  return set_params(p.data());
}

std::string Net::set_params(const float* host) {
  MLP_TRY(cudaMemcpyAsync(P_, host, sizeof(float) * NP, cudaMemcpyHostToDevice, stream_), "h2d");
  k_pack_weights<<<96, 256, 0, stream_>>>(P_, Wb_, WTb_);
  MLP_TRY(cudaGetLastError(), "pack");
  MLP_TRY(cudaMemsetAsync(M1_, 0, sizeof(float) * NP, stream_), "memset");
  MLP_TRY(cudaMemsetAsync(M2_, 0, sizeof(float) * NP, stream_), "memset");
  step_ = 0;
  MLP_TRY(cudaStreamSynchronize(stream_), "sync");
  return "";
}

std::string Net::get_params(float* host) {
  MLP_TRY(cudaMemcpyAsync(host, P_, sizeof(float) * NP, cudaMemcpyDeviceToHost, stream_), "d2h");
  MLP_TRY(cudaStreamSynchronize(stream_), "sync");
  return "";
}

int Net::num_params() { return NP; }

std::string Net::check_err() {
  int e = 0;
  MLP_TRY(cudaMemcpyAsync(&e, err_, sizeof(int), cudaMemcpyDeviceToHost, stream_), "d2h");
  MLP_TRY(cudaStreamSynchronize(stream_), "sync");
  if (e) {
    cudaMemsetAsync(err_, 0, sizeof(int), stream_);
    return "tensor-core wait timed out";
  }
  return "";
}

std::string Net::forward_dev(const __nv_bfloat16* X, int n, const int* n_dev, int max_n, float* y,
                             __nv_bfloat16* acts, cudaStream_t st) {
  const int grid = (max_n + TILE - 1) / TILE;
  if (grid <= 0) return "";
  k_mlp_fwd<<<grid, 128, fwd_smem(), st>>>(X, n, n_dev, Wb_, P_ + 3 * F * F, P_ + 3 * F * F + 3 * F,
                                            P_ + 3 * F * F + 4 * F, y, acts, err_);
  MLP_TRY(cudaGetLastError(), "mlp forward");
  return "";
}

std::string Net::backward_dev(const __nv_bfloat16* X, int n, const __nv_bfloat16* acts, const float* y,
                              const float* t, cudaStream_t st) {
  const int grid = (n + TILE - 1) / TILE;
  if (grid <= 0) return "";
  k_mlp_bwd<<<grid, 128, bwd_smem(), st>>>(X, n, WTb_, P_ + 3 * F * F + 4 * F - F, acts, y, t, 1.f / n, G_, err_);
  MLP_TRY(cudaGetLastError(), "mlp backward");
  return "";
}

std::string Net::predict(const float* Xh, int n, float* yh) {
  if (n <= 0) return "";
  std::vector<__nv_bfloat16> xb((size_t)n * F);
  for (size_t i = 0; i < xb.size(); ++i) xb[i] = __float2bfloat16_rn(Xh[i]);
  __nv_bfloat16* X = nullptr;
  float* y = nullptr;
  MLP_TRY(cudaMalloc(&X, sizeof(__nv_bfloat16) * xb.size()), "alloc");
  cudaError_t e = cudaMalloc(&y, sizeof(float) * n);
  if (e != cudaSuccess) { cudaFree(X); return std::string("alloc: ") + cudaGetErrorString(e); }
  std::string r;
  e = cudaMemcpyAsync(X, xb.data(), sizeof(__nv_bfloat16) * xb.size(), cudaMemcpyHostToDevice, stream_);
  if (e == cudaSuccess) r = forward_dev(X, n, nullptr, n, y, nullptr, stream_);
  else r = std::string("h2d: ") + cudaGetErrorString(e);
  if (r.empty()) {
    e = cudaMemcpyAsync(yh, y, sizeof(float) * n, cudaMemcpyDeviceToHost, stream_);
    if (e != cudaSuccess) r = std::string("d2h: ") + cudaGetErrorString(e);
  }
  cudaStreamSynchronize(stream_);
  cudaFree(X);
  cudaFree(y);
  if (r.empty()) r = check_err();
  return r;
}

std::string Net::gradients(const float* Xh, const float* th, int n, float* gh, float* loss) {
  if (n <= 0) return "empty batch";
  std::vector<__nv_bfloat16> xb((size_t)n * F);
  for (size_t i = 0; i < xb.size(); ++i) xb[i] = __float2bfloat16_rn(Xh[i]);
  std::vector<void*> tmp;
  auto fin = [&](const std::string& r) {
    cudaStreamSynchronize(stream_);
    for (void* p : tmp) cudaFree(p);
    return r;
  };
  __nv_bfloat16 *X = nullptr, *Aa = nullptr;
  float *y = nullptr, *t = nullptr;
  if (cudaMalloc(&X, sizeof(__nv_bfloat16) * xb.size()) != cudaSuccess) return fin("alloc");
  tmp.push_back(X);
  if (cudaMalloc(&Aa, sizeof(__nv_bfloat16) * 3 * (size_t)n * F) != cudaSuccess) return fin("alloc");
  tmp.push_back(Aa);
  if (cudaMalloc(&y, sizeof(float) * n) != cudaSuccess) return fin("alloc");
  tmp.push_back(y);
  if (cudaMalloc(&t, sizeof(float) * n) != cudaSuccess) return fin("alloc");
  tmp.push_back(t);
  cudaMemcpyAsync(X, xb.data(), sizeof(__nv_bfloat16) * xb.size(), cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(t, th, sizeof(float) * n, cudaMemcpyHostToDevice, stream_);
  cudaMemsetAsync(G_, 0, sizeof(float) * NG, stream_);
  std::string r = forward_dev(X, n, nullptr, n, y, Aa, stream_);
  if (r.empty()) r = backward_dev(X, n, Aa, y, t, stream_);
  if (!r.empty()) return fin(r);
  cudaMemcpyAsync(gh, G_, sizeof(float) * NP, cudaMemcpyDeviceToHost, stream_);
  float l = 0.f;
  cudaMemcpyAsync(&l, G_ + NP, sizeof(float), cudaMemcpyDeviceToHost, stream_);
  r = fin("");
  if (loss) *loss = l;
  if (r.empty()) r = check_err();
  return r;
}

std::string Net::train(const float* Xh, const float* th, int n, int epochs, int batch, float lr, float* last_loss) {
  if (n <= 0 || batch <= 0 || epochs <= 0) return "empty training set";
  std::vector<__nv_bfloat16> xb((size_t)n * F);
  for (size_t i = 0; i < xb.size(); ++i) xb[i] = __float2bfloat16_rn(Xh[i]);
  return train_dev_upload(xb.data(), th, n, epochs, batch, lr, last_loss);
}

std::string Net::train_dev_upload(const __nv_bfloat16* xb, const float* th, int n, int epochs, int batch, float lr,
                                  float* last_loss) {
  std::vector<void*> tmp;
  auto fin = [&](const std::string& r) {
    cudaStreamSynchronize(stream_);
    for (void* p : tmp) cudaFree(p);
    return r;
  };
  __nv_bfloat16 *X = nullptr, *Aa = nullptr;
  float *y = nullptr, *t = nullptr;
  const int bmax = batch < n ? batch : n;
  if (cudaMalloc(&X, sizeof(__nv_bfloat16) * (size_t)n * F) != cudaSuccess) return fin("alloc");
  tmp.push_back(X);
  if (cudaMalloc(&t, sizeof(float) * n) != cudaSuccess) return fin("alloc");
  tmp.push_back(t);
  if (cudaMalloc(&Aa, sizeof(__nv_bfloat16) * 3 * (size_t)bmax * F) != cudaSuccess) return fin("alloc");
  tmp.push_back(Aa);
  if (cudaMalloc(&y, sizeof(float) * bmax) != cudaSuccess) return fin("alloc");
  tmp.push_back(y);
  cudaMemcpyAsync(X, xb, sizeof(__nv_bfloat16) * (size_t)n * F, cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(t, th, sizeof(float) * n, cudaMemcpyHostToDevice, stream_);
  std::string r = train_device(X, t, n, epochs, batch, lr, Aa, y, last_loss);
  return fin(r);
}

std::string Net::train_device(const __nv_bfloat16* X, const float* t, int n, int epochs, int batch, float lr,
                              __nv_bfloat16* Aa, float* y, float* last_loss) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  double loss_sum = 0;
  int loss_cnt = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    loss_sum = 0;
    loss_cnt = 0;
    for (int s0 = 0; s0 < n; s0 += batch) {
      const int m = (n - s0) < batch ? (n - s0) : batch;
      MLP_TRY(cudaMemsetAsync(G_, 0, sizeof(float) * NG, stream_), "memset");
      const __nv_bfloat16* Xb = X + (size_t)s0 * F;
      std::string r = forward_dev(Xb, m, nullptr, m, y, Aa, stream_);
      if (r.empty()) r = backward_dev(Xb, m, Aa, y, t + s0, stream_);
      if (!r.empty()) return r;
      ++step_;
      const float c1 = 1.f / (1.f - std::pow(b1, (float)step_));
      const float c2 = 1.f / (1.f - std::pow(b2, (float)step_));
      k_adam<<<(NP + 255) / 256, 256, 0, stream_>>>(P_, G_, M1_, M2_, NP, lr, b1, b2, eps, c1, c2, Wb_, WTb_);
      MLP_TRY(cudaGetLastError(), "adam");
      float l = 0.f;
      MLP_TRY(cudaMemcpyAsync(&l, G_ + NP, sizeof(float), cudaMemcpyDeviceToHost, stream_), "d2h");
      MLP_TRY(cudaStreamSynchronize(stream_), "sync");
      loss_sum += l;
      ++loss_cnt;
    }
  }
  if (last_loss) *last_loss = loss_cnt ? (float)(loss_sum / loss_cnt) : 0.f;
  return check_err();
}

std::string Net::reserve_pairs(long long cap) {
  if (cap <= pair_cap_) return "";
  __nv_bfloat16* px = nullptr;
  float* pt = nullptr;
  MLP_TRY(cudaMalloc(&px, sizeof(__nv_bfloat16) * (size_t)cap * F), "alloc pairs");
  cudaError_t e = cudaMalloc(&pt, sizeof(float) * (size_t)cap);
  if (e != cudaSuccess) {
    cudaFree(px);
    return std::string("alloc pairs: ") + cudaGetErrorString(e);
  }
  if (!pair_count_) MLP_TRY(cudaMalloc(&pair_count_, sizeof(unsigned long long)), "alloc");
  long long have = 0;
  if (PX_) {
    have = num_pairs();
    if (have > 0) {
      cudaMemcpyAsync(px, PX_, sizeof(__nv_bfloat16) * (size_t)have * F, cudaMemcpyDeviceToDevice, stream_);
      cudaMemcpyAsync(pt, PT_, sizeof(float) * (size_t)have, cudaMemcpyDeviceToDevice, stream_);
    }
    cudaStreamSynchronize(stream_);
    cudaFree(PX_);
    cudaFree(PT_);
  }
  PX_ = px;
  PT_ = pt;
  pair_cap_ = cap;
  unsigned long long h = (unsigned long long)have;
  MLP_TRY(cudaMemcpyAsync(pair_count_, &h, sizeof(h), cudaMemcpyHostToDevice, stream_), "h2d");
  MLP_TRY(cudaStreamSynchronize(stream_), "sync");
  return "";
}

long long Net::num_pairs() {
  if (!pair_count_) return 0;
  unsigned long long h = 0;
  cudaMemcpyAsync(&h, pair_count_, sizeof(h), cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  return (long long)(h < (unsigned long long)pair_cap_ ? h : (unsigned long long)pair_cap_);
}

std::string Net::clear_pairs() {
  if (pair_count_) MLP_TRY(cudaMemsetAsync(pair_count_, 0, sizeof(unsigned long long), stream_), "memset");
  MLP_TRY(cudaStreamSynchronize(stream_), "sync");
  return "";
}

std::string Net::append_pairs(const __nv_bfloat16* X, const float* t, const int* n_dev, int max_n, cudaStream_t st,
                              long long* added) {
  if (added) *added = 0;
  if (!PX_) {
    std::string r = reserve_pairs(1LL << 22);
    if (!r.empty()) return r;
  }
  const long long before = num_pairs();
  // the solver's stream produced X and t: order this stream after it
  cudaEvent_t ev;
  MLP_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
  cudaEventRecord(ev, st);
  cudaStreamWaitEvent(stream_, ev, 0);
  cudaEventDestroy(ev);
  const int grid = (max_n + 255) / 256 < 4096 ? (max_n + 255) / 256 : 4096;
  k_append_pairs<<<grid > 0 ? grid : 1, 256, 0, stream_>>>(X, t, n_dev, PX_, PT_, pair_count_, pair_cap_);
  MLP_TRY(cudaGetLastError(), "append pairs");
  MLP_TRY(cudaStreamSynchronize(stream_), "sync");
  if (added) *added = num_pairs() - before;
  return "";
}

std::string Net::train_pairs(int epochs, int batch, float lr, unsigned long long seed, float* last_loss) {
  const long long n = num_pairs();
  if (n <= 0) return "no training pairs";
  if (n > 0x7fffffffLL) return "too many pairs";
  // one shuffle of the pairs, then epochs of sequential batches
  std::vector<int> perm((size_t)n);
  for (long long i = 0; i < n; ++i) perm[(size_t)i] = (int)i;
  std::mt19937_64 rng(seed);
  std::shuffle(perm.begin(), perm.end(), rng);
  std::vector<void*> tmp;
  auto fin = [&](const std::string& r) {
    cudaStreamSynchronize(stream_);
    for (void* p : tmp) cudaFree(p);
    return r;
  };
  int* dperm = nullptr;
  __nv_bfloat16 *Xs = nullptr, *Aa = nullptr;
  float *ts = nullptr, *y = nullptr;
  const int bmax = (long long)batch < n ? batch : (int)n;
  if (cudaMalloc(&dperm, sizeof(int) * (size_t)n) != cudaSuccess) return fin("alloc");
  tmp.push_back(dperm);
  if (cudaMalloc(&Xs, sizeof(__nv_bfloat16) * (size_t)n * F) != cudaSuccess) return fin("alloc");
  tmp.push_back(Xs);
  if (cudaMalloc(&ts, sizeof(float) * (size_t)n) != cudaSuccess) return fin("alloc");
  tmp.push_back(ts);
  if (cudaMalloc(&Aa, sizeof(__nv_bfloat16) * 3 * (size_t)bmax * F) != cudaSuccess) return fin("alloc");
  tmp.push_back(Aa);
  if (cudaMalloc(&y, sizeof(float) * bmax) != cudaSuccess) return fin("alloc");
  tmp.push_back(y);
  cudaMemcpyAsync(dperm, perm.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, stream_);
  k_gather_pairs<<<4096, 256, 0, stream_>>>(PX_, PT_, dperm, n, Xs, ts);
  if (cudaGetLastError() != cudaSuccess) return fin("gather pairs");
  return fin(train_device(Xs, ts, (int)n, epochs, batch, lr, Aa, y, last_loss));
}

}  // namespace mlp
}  // namespace lsgb
