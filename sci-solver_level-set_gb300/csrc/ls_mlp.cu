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


}  // namespace

// ---------------------------------------------------------------------------
// Weight copies for the tensor cores: BF16 tiles in the operand layout above
// (tile_off), so that one bulk asynchronous copy of 32 KB stages a layer's
// weights.  Wt[l]: rows = output feature, K = input feature (B operand of
// the forward); WTt[l]: rows = input feature, K = output feature (B operand
// of the backward's dH = d W).
__device__ __forceinline__ void store_weight(__nv_bfloat16* Wt, __nv_bfloat16* WTt, int i, float p) {
  const int l = i / (F * F), o = (i / F) % F, in = i % F;
  const __nv_bfloat16 v = __float2bfloat16_rn(p);
  Wt[(size_t)l * F * F + tile_off(o, in) / 2] = v;
  WTt[(size_t)l * F * F + tile_off(in, o) / 2] = v;
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// one tile (32 KB, 16-byte aligned at both ends) from global into shared
// memory, completing on bar
__device__ __forceinline__ void bulk_tile(uint8_t* dst, const __nv_bfloat16* src, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(__cvta_generic_to_global(src)), "r"((uint32_t)TILE_BYTES), "r"(smem_u32(bar))
               : "memory");
}

// MMAs of one 128 x 128 x 128 product that add to the accumulator when acc
// is set (thread 0 only)
__device__ __forceinline__ void mma_tile_acc(uint32_t tmem_d, const uint8_t* a, const uint8_t* b, bool acc) {
  const uint32_t sa = smem_u32(a), sb = smem_u32(b);
#pragma unroll
  for (int ks = 0; ks < F / 16; ++ks)
    mma(tmem_d, make_desc(sa + ks * 2 * LBO), make_desc(sb + ks * 2 * LBO), (acc || ks > 0) ? 1 : 0);
}

struct SmemW {
  uint64_t bar;    // MMA completion
  uint64_t bar_w;  // weight tiles staged
  uint32_t tmem;
  int fail;
};

// ---------------------------------------------------------------------------
// Forward.  X [n][128] BF16 rows; Wt the three weight tiles; b [3][128],
// w4 [128], b4 [1] fp32; y [n]; A (optional) [3][n][128] BF16 activations
// a_1..a_3 for the backward pass.  n_dev (optional) overrides n from device
// memory (graph replays with a device-side sample count).  Each CTA stages
// the weights once (three bulk copies) and then runs the sample tiles
// blockIdx.x, blockIdx.x + gridDim.x, ... through the three layers.
__global__ void __launch_bounds__(128, 1)
    k_mlp_fwd(const __nv_bfloat16* __restrict__ X, int n, const int* n_dev, const __nv_bfloat16* __restrict__ Wt,
              const float* __restrict__ b, const float* __restrict__ w4, const float* __restrict__ b4,
              float* __restrict__ y, __nv_bfloat16* __restrict__ A, int* err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* act = base;                       // activation tile (A operand)
  uint8_t* wt = base + TILE_BYTES;           // 3 weight tiles (B operands)
  SmemW* sm = reinterpret_cast<SmemW*>(base + 4 * TILE_BYTES);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (n_dev) n = *n_dev;
  const int ntiles = (n + TILE - 1) / TILE;
  if ((int)blockIdx.x >= ntiles) return;  // whole CTA exits before any tensor-core work
  if (tid == 0) {
    mbar_init(&sm->bar, 1);
    mbar_init(&sm->bar_w, 1);
    sm->fail = 0;
    mbar_expect_tx(&sm->bar_w, 3 * TILE_BYTES);
    for (int l = 0; l < 3; ++l) bulk_tile(wt + l * TILE_BYTES, Wt + (size_t)l * F * F, &sm->bar_w);
  }
  __syncwarp();
  if (warp == 0) tmem_alloc(&sm->tmem, 128);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = sm->tmem;
  uint32_t phase = 0;
  bool ok = true, weights = false, mma_pending = false;
  for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int s0 = tile * TILE;
    const int s = s0 + tid;  // sample row tid of the operand tile
    if (s < n) load_row(act, tid, X + (size_t)s * F);
    else zero_row(act, tid);
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    if (!weights) {
      ok = __syncthreads_and(mbar_wait(&sm->bar_w, 0)) != 0;
      weights = ok;
      if (!ok) break;
    }
    float out = 0.f;
    for (int l = 0; l < 3 && ok; ++l) {
      if (tid == 0) {
        mma_tile_acc(tmem, act, wt + l * TILE_BYTES, false);
        mma_commit(&sm->bar);
      }
      mma_pending = true;
      ok = __syncthreads_and(mbar_wait(&sm->bar, phase)) != 0;
      if (!ok) break;
      mma_pending = false;
      phase ^= 1;
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
    }
  }
  if (!ok) {
    sm->fail = 1;
    if (err) atomicExch(err, 1);
    // drain (bounded): the weight copies and the MMAs in flight before TMEM goes
    if (!weights) mbar_wait(&sm->bar_w, 0);
    if (mma_pending) mbar_wait(&sm->bar, phase);
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0) tmem_dealloc(tmem, 128);
}

// ---------------------------------------------------------------------------
// Backward.  Each CTA runs the sample tiles blockIdx.x, blockIdx.x +
// gridDim.x, ...; the three weight gradients accumulate in tensor memory
// across its tiles (gW_l in columns [128 l, 128 l + 128), the back-propagated
// dH of the current layer in [384, 512)); the bias, w4 and b4 gradients and
// the loss accumulate in shared memory and registers.  At the end the CTA
// writes its sums as row blockIdx.x of Gp [gridDim.x][NG_STRIDE], laid out as G =
// [gW (3x128x128) | gb (3x128) | gw4 (128) | gb4 (1) | loss (1)]; k_mlp_reduce
// adds the rows in a fixed order (no atomics in global memory, the same
// gradient bits on every run).  WTt: the transposed weight tiles (layers 1
// and 2 are staged once per CTA by bulk copies); A the forward activations;
// t the targets.
constexpr int NG_ROW = 3 * F * F + 3 * F + F + 1 + 1;
// rows of Gp start on 16-byte boundaries (the weight gradients are stored as
// float4)
constexpr int NG_STRIDE = (NG_ROW + 3) & ~3;

__global__ void __launch_bounds__(128, 1)
    k_mlp_bwd(const __nv_bfloat16* __restrict__ X, int n, const __nv_bfloat16* __restrict__ WTt,
              const float* __restrict__ w4, const __nv_bfloat16* __restrict__ A, const float* __restrict__ y,
              const float* __restrict__ t, float inv_n, float* __restrict__ Gp, int* err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* dT = base;                   // A operand of gW: d^T  (rows = out, K = samples)
  uint8_t* aT = base + TILE_BYTES;      // B operand of gW: a^T  (rows = in,  K = samples)
  uint8_t* dN = base + 2 * TILE_BYTES;  // A operand of dH: d    (rows = samples, K = out)
  uint8_t* wN1 = base + 3 * TILE_BYTES;  // B operand of dH for layer 1: W_1^T (rows = in, K = out)
  uint8_t* wN2 = base + 4 * TILE_BYTES;  // the same for layer 2
  // bias and w4 gradients, each entry owned by one thread (fixed summation
  // order: the gradients come out the same on every run)
  float* s_gb = reinterpret_cast<float*>(base + 5 * TILE_BYTES);  // [3][128] bias gradients
  float* s_gw4 = s_gb + 3 * F;                                     // [128]
  float* s_gw4w = s_gw4 + F;                                       // [4][128] the tile's per-warp w4 sums
  float* s_red = s_gw4w + 4 * F;                                   // [2][4] per-warp gb4 and loss
  SmemW* sm = reinterpret_cast<SmemW*>(s_red + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntiles = (n + TILE - 1) / TILE;
  if ((int)blockIdx.x >= ntiles) return;
  if (tid == 0) {
    mbar_init(&sm->bar, 1);
    mbar_init(&sm->bar_w, 1);
    sm->fail = 0;
    mbar_expect_tx(&sm->bar_w, 2 * TILE_BYTES);
    bulk_tile(wN1, WTt + (size_t)1 * F * F, &sm->bar_w);
    bulk_tile(wN2, WTt + (size_t)2 * F * F, &sm->bar_w);
  }
  for (int i = tid; i < 4 * F; i += blockDim.x) s_gb[i] = 0.f;  // s_gb and s_gw4
  __syncwarp();
  if (warp == 0) tmem_alloc(&sm->tmem, 512);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tm = sm->tmem;
  const int r = tid;                // sample row of this thread in the operand phase
  const int rr = warp * 32 + lane;  // accumulator row of this thread (the same index)
  const uint32_t trow = tm + ((uint32_t)(warp * 32) << 16);
  float gb4_acc = 0.f, loss_acc = 0.f;
  uint32_t phase = 0;
  bool ok = true, weights = false, mma_pending = false, first = true;
  for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int s0 = tile * TILE;
    const int s = s0 + r;
    const bool valid = s < n;
    // output layer
    float dy = 0.f;
    if (valid) {
      const float e = y[s] - t[s];
      dy = e * inv_n;
      loss_acc += 0.5f * e * e * inv_n;
    }
    gb4_acc += dy;
    // d_3 = bf16(dy w4 [a_3 > 0]); its column sums are gb_3
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
      for (int j = 0; j < 8; ++j) dv[j] = bf16r(av[j] > 0.f ? dy * __ldg(w4 + c + j) : 0.f);
      *reinterpret_cast<uint4*>(dN + tile_off(r, c)) = pack8(dv);
#pragma unroll
      for (int j = 0; j < 8; ++j) *reinterpret_cast<__nv_bfloat16*>(dT + tile_off(c + j, r)) = __float2bfloat16_rn(dv[j]);
    }
    // gw4[j] += sum_r dy_r a3[r][j]: warp sums through shuffles, added up
    // per column after the next barrier
    for (int c = 0; c < F; ++c) {
      float v = valid ? dy * __bfloat162float(a3[c]) : 0.f;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) s_gw4w[warp * F + c] = v;
    }
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
      fence_async_smem();
      fence_before();
      __syncthreads();
      fence_after();
      if (!weights) {
        ok = __syncthreads_and(mbar_wait(&sm->bar_w, 0)) != 0;
        weights = ok;
        if (!ok) break;
      }
      // gb_l: thread tid sums row tid of d^T (the tile's samples in order;
      // padding samples are zero); the tensor cores only read dT meanwhile
      {
        float sum = 0.f;
        for (int k = 0; k < TILE; k += 8) {
          const uint4 raw = *reinterpret_cast<const uint4*>(dT + tile_off(tid, k));
          const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&raw);
#pragma unroll
          for (int j = 0; j < 8; ++j) sum += __bfloat162float(hb[j]);
        }
        s_gb[l * F + tid] += sum;
        if (l == 2) s_gw4[tid] += (s_gw4w[tid] + s_gw4w[F + tid]) + (s_gw4w[2 * F + tid] + s_gw4w[3 * F + tid]);
      }
      if (tid == 0) {
        mma_tile_acc(tm + l * 128, dT, aT, !first);                   // gW_l (+)= d_l^T a_{l-1}
        if (l > 0) mma_tile_acc(tm + 384, dN, l == 2 ? wN2 : wN1, false);  // dH = d_l W_l
        mma_commit(&sm->bar);
      }
      mma_pending = true;
      ok = __syncthreads_and(mbar_wait(&sm->bar, phase)) != 0;
      if (!ok) break;
      mma_pending = false;
      phase ^= 1;
      fence_after();
      if (l > 0) {
        // d_{l-1} for sample rr = bf16(dH * [a_{l-1} > 0]); its column sums are gb_{l-1}
        const int sr = s0 + rr;
        const bool vr = sr < n;
        const __nv_bfloat16* ap = A + ((size_t)(l - 1) * n + (vr ? sr : s0)) * F;
        for (int c = 0; c < F / 32; ++c) {
          float v[32];
          tmem_ld32(trow + 384 + c * 32, v);
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const float a = vr ? __bfloat162float(ap[c * 32 + j]) : 0.f;
            v[j] = bf16r(a > 0.f ? v[j] : 0.f);
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) *reinterpret_cast<uint4*>(dN + tile_off(rr, c * 32 + q * 8)) = pack8(v + q * 8);
#pragma unroll
          for (int j = 0; j < 32; ++j)
            *reinterpret_cast<__nv_bfloat16*>(dT + tile_off(c * 32 + j, rr)) = __float2bfloat16_rn(v[j]);
        }
      }
      fence_before();
      __syncthreads();
      fence_after();
    }
    first = false;
  }
  if (ok) {
    float* row = Gp + (size_t)blockIdx.x * NG_STRIDE;
    // weight gradients: row rr of each gW_l from tensor memory
    for (int l = 0; l < 3; ++l)
      for (int c = 0; c < F / 32; ++c) {
        float v[32];
        tmem_ld32(trow + l * 128 + c * 32, v);
        float4* dst = reinterpret_cast<float4*>(row + ((size_t)l * F + rr) * F + c * 32);
#pragma unroll
        for (int q = 0; q < 8; ++q) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      }
    for (int o = 16; o > 0; o >>= 1) {
      gb4_acc += __shfl_xor_sync(0xffffffffu, gb4_acc, o);
      loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
    }
    if (lane == 0) {
      s_red[warp] = gb4_acc;
      s_red[4 + warp] = loss_acc;
    }
    __syncthreads();
    for (int i = tid; i < 4 * F; i += blockDim.x) row[3 * F * F + i] = s_gb[i];  // gb and gw4
    if (tid == 0) {
      row[3 * F * F + 4 * F] = (s_red[0] + s_red[1]) + (s_red[2] + s_red[3]);
      row[3 * F * F + 4 * F + 1] = (s_red[4] + s_red[5]) + (s_red[6] + s_red[7]);
    }
  } else {
    sm->fail = 1;
    if (err) atomicExch(err, 1);
    if (!weights) mbar_wait(&sm->bar_w, 0);
    if (mma_pending) mbar_wait(&sm->bar, phase);
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0) tmem_dealloc(sm->tmem, 512);
}

// G[i] = sum over the rows of Gp (fixed order); the loss of the batch is
// also added to *loss_acc when it is given (the epoch's sum on the device).
__global__ void k_mlp_reduce(const float* __restrict__ Gp, int rows, float* __restrict__ G, float* loss_acc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NG_ROW; i += gridDim.x * blockDim.x) {
    float sum = 0.f;
    for (int r = 0; r < rows; ++r) sum += Gp[(size_t)r * NG_STRIDE + i];
    G[i] = sum;
    if (loss_acc && i == NG_ROW - 1) *loss_acc += sum;
  }
}

// ---------------------------------------------------------------------------
// Adam on the fp32 master parameters P = [W (3x128x128) | b (3x128) | w4 |
// b4]; refreshes the BF16 weight tiles.
__global__ void k_adam(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M1,
                       float* __restrict__ M2, int np, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16* __restrict__ Wt, __nv_bfloat16* __restrict__ WTt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const float g = G[i];
    const float m = b1 * M1[i] + (1.f - b1) * g;
    const float v = b2 * M2[i] + (1.f - b2) * g * g;
    M1[i] = m;
    M2[i] = v;
    const float p = P[i] - lr * (m * c1) / (sqrtf(v * c2) + eps);
    P[i] = p;
    if (i < 3 * F * F) store_weight(Wt, WTt, i, p);
  }
}

__global__ void k_pack_weights(const float* __restrict__ P, __nv_bfloat16* __restrict__ Wt,
                               __nv_bfloat16* __restrict__ WTt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * F * F; i += gridDim.x * blockDim.x)
    store_weight(Wt, WTt, i, P[i]);
}

// ---------------------------------------------------------------------------
// Features of the vertices in vlist (product vertex ids): slot 0 = the vertex
// itself (0, 0, 0, phi / h), slots 1..31 = its first 31 1-ring neighbours
// (ascending id) as (dx, dy, dz, phi) / h, zeros beyond the ring.  h is
// 1 / inv_h, or 1 / vinv_h[v] per vertex when given (batches of meshes of
// different resolution).
__global__ void k_features(int nlist, const int* __restrict__ vlist, const int* __restrict__ nlist_dev,
                           const int* __restrict__ adj_off, const int* __restrict__ adj, const float* __restrict__ xyz,
                           int nv, const float* __restrict__ phi, float inv_h, const float* __restrict__ vinv_h,
                           __nv_bfloat16* __restrict__ Xo) {
  if (nlist_dev) nlist = *nlist_dev;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nlist; i += gridDim.x * blockDim.x) {
    const int v = vlist[i];
    if (vinv_h) inv_h = vinv_h[v];
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
static_assert(NG == NG_ROW, "gradient row layout");
size_t fwd_smem() { return 4 * (size_t)TILE_BYTES + 1024 + 64; }
size_t bwd_smem() { return 5 * (size_t)TILE_BYTES + (8 * F + 8) * sizeof(float) + 1024 + 64; }
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
  MLP_TRY(alloc((void**)&loss_acc_, sizeof(float)), "alloc");
  {
    int dev = 0;
    MLP_TRY(cudaGetDevice(&dev), "device");
    MLP_TRY(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev), "device");
    if (sms_ < 1) sms_ = 1;
  }
  // one partial-gradient row per backward CTA (at most one CTA per SM)
  MLP_TRY(alloc((void**)&Gp_, sizeof(float) * (size_t)NG_STRIDE * sms_), "alloc");
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
  // one CTA per SM at most, each over several sample tiles (the weights are
  // staged once per CTA)
  const int tiles = (max_n + TILE - 1) / TILE;
  const int grid = tiles < sms_ ? tiles : sms_;
  if (grid <= 0) return "";
  k_mlp_fwd<<<grid, 128, fwd_smem(), st>>>(X, n, n_dev, Wb_, P_ + 3 * F * F, P_ + 3 * F * F + 3 * F,
                                            P_ + 3 * F * F + 4 * F, y, acts, err_);
  MLP_TRY(cudaGetLastError(), "mlp forward");
  return "";
}

std::string Net::backward_dev(const __nv_bfloat16* X, int n, const __nv_bfloat16* acts, const float* y,
                              const float* t, cudaStream_t st, float* loss_sink) {
  const int tiles = (n + TILE - 1) / TILE;
  const int grid = tiles < sms_ ? tiles : sms_;
  if (grid <= 0) return "";
  k_mlp_bwd<<<grid, 128, bwd_smem(), st>>>(X, n, WTb_, P_ + 3 * F * F + 4 * F - F, acts, y, t, 1.f / n, Gp_, err_);
  MLP_TRY(cudaGetLastError(), "mlp backward");
  k_mlp_reduce<<<(NG + 255) / 256, 256, 0, st>>>(Gp_, grid, G_, loss_sink);
  MLP_TRY(cudaGetLastError(), "mlp gradient reduction");
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
  float loss_sum = 0.f;
  int loss_cnt = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    // the batches' losses add up on the device; one read per epoch
    MLP_TRY(cudaMemsetAsync(loss_acc_, 0, sizeof(float), stream_), "memset");
    loss_cnt = 0;
    for (int s0 = 0; s0 < n; s0 += batch) {
      const int m = (n - s0) < batch ? (n - s0) : batch;
      const __nv_bfloat16* Xb = X + (size_t)s0 * F;
      std::string r = forward_dev(Xb, m, nullptr, m, y, Aa, stream_);
      if (r.empty()) r = backward_dev(Xb, m, Aa, y, t + s0, stream_, loss_acc_);
      if (!r.empty()) return r;
      ++step_;
      const float c1 = 1.f / (1.f - std::pow(b1, (float)step_));
      const float c2 = 1.f / (1.f - std::pow(b2, (float)step_));
      k_adam<<<(NP + 255) / 256, 256, 0, stream_>>>(P_, G_, M1_, M2_, NP, lr, b1, b2, eps, c1, c2, Wb_, WTb_);
      MLP_TRY(cudaGetLastError(), "adam");
      ++loss_cnt;
    }
    MLP_TRY(cudaMemcpyAsync(&loss_sum, loss_acc_, sizeof(float), cudaMemcpyDeviceToHost, stream_), "d2h");
    MLP_TRY(cudaStreamSynchronize(stream_), "sync");
    std::string r = check_err();
    if (!r.empty()) return r;
  }
  if (last_loss) *last_loss = loss_cnt ? loss_sum / loss_cnt : 0.f;
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

std::string Net::eval_pairs(long long first, long long count, float* abs_err) {
  const long long n = num_pairs();
  if (first < 0 || count < 0 || first + count > n) return "pair range outside the buffer";
  if (count == 0) return "";
  if (count > 0x7fffffffLL) return "too many pairs";
  float* y = nullptr;
  MLP_TRY(cudaMalloc(&y, sizeof(float) * (size_t)count), "alloc");
  std::string r = forward_dev(PX_ + (size_t)first * F, (int)count, nullptr, (int)count, y, nullptr, stream_);
  std::vector<float> yh((size_t)count), th((size_t)count);
  if (r.empty() &&
      (cudaMemcpyAsync(yh.data(), y, sizeof(float) * (size_t)count, cudaMemcpyDeviceToHost, stream_) != cudaSuccess ||
       cudaMemcpyAsync(th.data(), PT_ + first, sizeof(float) * (size_t)count, cudaMemcpyDeviceToHost, stream_) !=
           cudaSuccess))
    r = "d2h";
  cudaStreamSynchronize(stream_);
  cudaFree(y);
  if (!r.empty()) return r;
  for (long long i = 0; i < count; ++i) abs_err[i] = std::fabs(yh[(size_t)i] - th[(size_t)i]);
  return check_err();
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
