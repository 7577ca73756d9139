// gemm_api.h -- batched BF16 tcgen05 GEMM and operand packing.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace pysa_gb {

struct GemmArgs {
  const uint16_t* A;  // packed [batch][M/128][K/64] tiles of 128 x 64
  const uint16_t* B;  // packed [batch][N/256][K/64] tiles of 256 x 64
  float* C;           // [batch][M][ldc]
  const float* bias;  // [batch][N] or null
  int32_t* status;
  int64_t strideA, strideB, strideC, strideBias;  // elements per batch item
  int32_t M, N, K, ldc;
  int32_t accumulate;  // C += A B^T
  int32_t relu;        // ReLU after bias
};

cudaError_t launch_gemm_tc(const GemmArgs& g, int batch, cudaStream_t st);
cudaError_t launch_pack_kmajor(const float* src, int ld, int64_t src_stride,
                               int rows, int K, int transpose, int tile_rows,
                               uint16_t* dst, int64_t dst_stride, int batch,
                               cudaStream_t st);

}  // namespace pysa_gb
