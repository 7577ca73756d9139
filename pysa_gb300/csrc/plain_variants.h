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

// Per-variant constants for building the work list on the device.
struct PlainItemPlan {
  int nc[kNumPlainVariants];          // columns per lane (n <= 32 nc)
  int cpb[kNumPlainVariants];         // chains per work item
  int row_floats[kNumPlainVariants];  // floats per packed coupling row
  int start[kNumPlainVariants];       // first work item of each variant
  __host__ __device__ int variant_of(int n) const {
    for (int v = 0; v < kNumPlainVariants; ++v)
      if (n <= 32 * nc[v]) return v;
    return kNumPlainVariants - 1;
  }
};
PlainItemPlan make_item_plan();

// Records `msg` as the calling thread's last error and returns `code`.
int pysa_gb_internal_fail(int code, const char* msg);

}  // namespace pysa_gb
