// csr_api.h -- host interface of the sparse-row Metropolis sweep.
#pragma once
#include <cuda_runtime.h>

#include "../../include/pysa_gb.h"

namespace pysa_gb {

struct SweepItem;

// Most chains per CTA of the sparse-row sweep (one thread per chain).
constexpr int kCsrChains = 128;

struct CsrArgs {
  pysa_gb_problems p;
  pysa_gb_state s;
  const int32_t* perm;
  int32_t perm_slots;
  int32_t num_items;
  const SweepItem* items;
  uint64_t seed;
  int32_t width;   // 0: grouped rows; 4/8/16/32: fixed records
  int32_t chains;  // chains per work item = threads per CTA (<= kCsrChains)
};

// One sweep of every work item (a CTA each).
cudaError_t launch_csr(const CsrArgs& a, bool random, cudaStream_t st);

}  // namespace pysa_gb
