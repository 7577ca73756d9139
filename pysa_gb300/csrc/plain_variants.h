// plain_variants.h -- compile-time variants of the plain sweep kernel.
// A variant is picked by the instance size: NC = columns per lane
// (n <= 32 NC), GW = chains per warp, W = warps per CTA, RB = ring rows.
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

namespace pysa_gb {

struct PlainArgs;

struct PlainVariant {
  int nc, gw, w, rb;
  // launch one sweep over `items` work items; returns the CUDA error
  cudaError_t (*launch)(const PlainArgs&, bool random, int grid,
                        cudaStream_t st);
  size_t (*smem)(bool random);
  const void* (*func)(bool random);
};

constexpr int kNumPlainVariants = 8;
const PlainVariant& plain_variant(int v);
int plain_variant_for(int n);  // -1 if n is too large

}  // namespace pysa_gb
