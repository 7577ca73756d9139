// wide_api.h -- host interface of the plain sweep for dense instances wider
// than the register-resident kernel's limit.
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

#include "../../include/pysa_gb.h"

namespace pysa_gb {

struct SweepItem;

// Instances with more spins than this take k_sweep_wide.
constexpr int kPlainMaxN = 4096;
// Chains per CTA of k_sweep_wide (one warp each).
constexpr int kWideWarps = 8;

struct WideArgs {
  pysa_gb_problems p;
  pysa_gb_state s;
  const int32_t* perm;
  float* fields;
  int32_t field_ld;
  int32_t perm_slots;
  const SweepItem* items;
  int32_t num_items;
  int32_t pad_;
  uint64_t seed;
};

// Shared memory of one CTA: the spin words of its chains.
size_t wide_smem_bytes(int words);
// One sweep of every work item (kWideWarps chains each), at most max_ctas
// CTAs looping over the items.
cudaError_t launch_wide(const WideArgs& a, bool random, int max_ctas,
                        cudaStream_t st);

}  // namespace pysa_gb
