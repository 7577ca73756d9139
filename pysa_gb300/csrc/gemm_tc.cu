// gemm_tc.cu -- batched BF16 GEMM on the 5th-generation tensor cores for the
// learned flip proposal (MLP forward, backward and weight gradients).
//
//   C[b] (+)= A[b] * B[b]^T (+ bias[b], optionally ReLU), FP32 accumulation
//
// A is M x K and B is N x K, both BF16 and pre-packed by k_pack_kmajor into
// the canonical no-swizzle K-major core-matrix layout: tiles of 128 (A) or
// 256 (B) rows by 64 K, 16 KB / 32 KB each, so one 1-D bulk copy (TMA
// engine) moves a whole MMA operand tile.  One CTA computes a 128 x 256
// output tile in tensor memory: warp 5 streams the A/B tiles through a ring of
// shared-memory stages, one thread of warp 4 issues the tcgen05.mma
// instructions (four K=16 steps per 64-wide K tile) and warps 0-3 (thread =
// TMEM lane = output row) read the accumulator back with tcgen05.ld, add the
// bias, apply the ReLU and store FP32 rows.  M must be a multiple of 128, N of
// 256 and K of 64.  Every wait is bounded.
#include "aux.cuh"
#include "gemm_api.h"
#include "tc_ptx.cuh"

namespace pysa_gb {

namespace {
constexpr int kStages = 4;
constexpr uint32_t kATile = 16384, kBTile = 32768;
constexpr uint32_t kStage = kATile + kBTile;
constexpr size_t kBarOff = (size_t)kStages * kStage;
constexpr size_t kSmem = kBarOff + (2 * kStages + 1) * 8 + 16;

__device__ __forceinline__ bool gwait(uint64_t* bar, uint32_t parity,
                                      int32_t* status) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (globaltimer_ns() - t0 > 1000000000ull) {
      set_status(status, PYSA_GB_ERR_TIMEOUT);
      return false;
    }
  }
}
}  // namespace

__global__ void __launch_bounds__(192, 1) k_gemm_tc(const GemmArgs g) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kBarOff);
  uint64_t* empty = full + kStages;
  uint64_t* done = empty + kStages;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x, nt = blockIdx.y, b = blockIdx.z;
  const int kt_n = g.K / 64;
  const uint16_t* A = g.A + (size_t)b * g.strideA +
                      (size_t)mt * kt_n * (kATile / 2);
  const uint16_t* B = g.B + (size_t)b * g.strideB +
                      (size_t)nt * kt_n * (kBTile / 2);

  if (warp == 0) {
    tc::tmem_alloc(tslot, 256);
    tc::tmem_relinquish();
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *tslot;
  const uint32_t sbase = smem_addr(smem);

  if (warp == 5 && lane == 0) {
    int issued = 0;
    for (int kt = 0; kt < kt_n; ++kt) {
      const int s = kt % kStages;
      if (kt >= kStages &&
          !gwait(&empty[s], ((kt / kStages) - 1) & 1, g.status))
        break;
      mbar_expect_tx_arrive(&full[s], kStage);
      bulk_g2s(smem + s * kStage, A + (size_t)kt * (kATile / 2), kATile,
               &full[s]);
      bulk_g2s(smem + s * kStage + kATile, B + (size_t)kt * (kBTile / 2),
               kBTile, &full[s]);
      issued = kt + 1;
    }
    // the CTA stays until its last copies have landed (bounded)
    for (int kt = issued > kStages ? issued - kStages : 0; kt < issued; ++kt)
      gwait(&full[kt % kStages], (kt / kStages) & 1, g.status);
  } else if (warp == 4 && lane == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, 256);
    bool ok = true;
    for (int kt = 0; kt < kt_n; ++kt) {
      const int s = kt % kStages;
      if (!gwait(&full[s], (kt / kStages) & 1, g.status)) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const uint32_t a0 = sbase + s * kStage, b0 = a0 + kATile;
#pragma unroll
      for (int ks = 0; ks < 4; ++ks)
        tc::mma_bf16(taddr, tc::smem_desc(a0 + 256 * ks, 128, 1024),
                     tc::smem_desc(b0 + 256 * ks, 128, 1024), idesc,
                     (kt | ks) ? 1u : 0u);
      tc::commit(&empty[s]);
    }
    if (ok) tc::commit(done);
  } else if (warp < 4) {
    const bool ok = gwait(done, 0, g.status);
    tc::fence_after_sync();
    if (__all_sync(0xffffffffu, ok)) {
      const int row = mt * 128 + warp * 32 + lane;
      float* C = g.C + (size_t)b * g.strideC + (size_t)row * g.ldc;
      const float* bias =
          g.bias ? g.bias + (size_t)b * g.strideBias + nt * 256 : nullptr;
      for (int c0 = 0; c0 < 256; c0 += 32) {
        float v[32];
        tc::tmem_ld32(taddr + ((uint32_t)(warp * 32) << 16) + c0, v);
        float* out = C + nt * 256 + c0;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          float x = v[i];
          if (bias) x += bias[c0 + i];
          if (g.accumulate) x += out[i];
          if (g.relu) x = fmaxf(x, 0.0f);
          out[i] = x;
        }
      }
    }
  }
  __syncwarp();
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(taddr, 256);
  }
}

// Pack rows x K of an FP32 matrix into BF16 K-major core-matrix tiles of
// `tile_rows` rows (128 or 256) by 64.  src(r, k) = src[r * ld + k], or
// src[k * ld + r] when `transpose`.  Batched over blockIdx.y.
__global__ void k_pack_kmajor(const float* src, int ld, int64_t src_stride,
                              int rows, int K, int transpose, int tile_rows,
                              uint16_t* dst, int64_t dst_stride) {
  const int64_t total = (int64_t)rows * K;
  const float* s = src + (size_t)blockIdx.y * src_stride;
  uint16_t* d = dst + (size_t)blockIdx.y * dst_stride;
  const int kt_n = K / 64;
  const int64_t tile = (int64_t)tile_rows * 64;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = e / tile;
    const int within = (int)(e % tile);
    const int rt = (int)(t / kt_n), kt = (int)(t % kt_n);
    const int cm = within / 64, inside = within % 64;
    const int r = rt * tile_rows + (cm / 8) * 8 + inside / 8;
    const int k = kt * 64 + (cm % 8) * 8 + inside % 8;
    const float v = transpose ? s[(int64_t)k * ld + r] : s[(int64_t)r * ld + k];
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    d[e] = *reinterpret_cast<const uint16_t*>(&h);
  }
}

cudaError_t launch_gemm_tc(const GemmArgs& g, int batch, cudaStream_t st) {
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(
        k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  dim3 grid(g.M / 128, g.N / 256, batch);
  k_gemm_tc<<<grid, 192, kSmem, st>>>(g);
  return cudaGetLastError();
}

cudaError_t launch_pack_kmajor(const float* src, int ld, int64_t src_stride,
                               int rows, int K, int transpose, int tile_rows,
                               uint16_t* dst, int64_t dst_stride, int batch,
                               cudaStream_t st) {
  const int64_t total = (int64_t)rows * K;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  dim3 grid(blocks, batch);
  k_pack_kmajor<<<grid, 256, 0, st>>>(src, ld, src_stride, rows, K, transpose,
                                      tile_rows, dst, dst_stride);
  return cudaGetLastError();
}

}  // namespace pysa_gb
