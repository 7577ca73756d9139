// tc_api.h -- argument blocks of the tensor-core blocked sweep.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/pysa_gb.h"

namespace pysa_gb {

struct TcItem {
  int32_t inst, chain0, nchains, fold;
  int64_t b_off;     // element offset into the packed BF16 tiles
  int64_t diag_off;  // element offset into the packed FP32 diagonal blocks
};

struct TcArgs {
  pysa_gb_problems p;
  pysa_gb_state s;
  float* fields;
  int32_t field_ld;
  int32_t terms;  // 1: J exact in BF16; 2: J_hi + J_lo
  const uint16_t* tc_b;
  const float* tc_diag;
  const TcItem* items;
  uint64_t seed;
  int32_t recompute_every;  // >0: H and E rebuilt when sweep % this == 0
  int32_t pad_;
  // optional timeline of CTA 0 (globaltimer ns): [block][8] stamps
  unsigned long long* trace;
};

int tc_fold_for(int n);  // 1, 2, 4 or -1 (n > 2048)
int tc_chains_per_cta(int n);
int64_t tc_b_elems(int n, int terms);
int64_t tc_diag_elems(int n);
cudaError_t launch_pack_tc(const float* Jt, int ld, int n, int terms,
                           uint16_t* b_out, float* diag_out, cudaStream_t st);
cudaError_t launch_tc(const TcArgs& a, int F, int count, cudaStream_t st);

}  // namespace pysa_gb
