// ais_api.h -- argument blocks of the AIS and exact log-Z kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pysa_gb {

// Instance b = blockIdx.y; its samples are its reads (one replica each),
// chains chain_off[b] .. + reads[b] - 1.
struct AisArgs {
  int32_t problem_type, words, num_temps, update, ref, order, max_n,
      num_instances;
  double p;
  uint64_t seed;
  const int32_t* n_tab;
  const int32_t* ld_tab;
  const int32_t* replicas;
  const int32_t* reads;
  const int64_t* j_off;
  const int64_t* chain_off;
  const float* J;        // transposed couplings (row i = field change of i)
  const float* temps;    // [num_temps] anneal schedule
  const int32_t* perm;   // [num_temps, num_instances, max_n] orders (random)
  const float* fields;   // [chains, field_ld] initial local fields
  int32_t field_ld;
  int32_t pad_;
  uint32_t* spins;       // [chains, words] in/out
  float* energies;       // [chains] in/out
  double* log_w;         // [chains] out
  int32_t* status;       // set when an instance has more than one replica
};

struct LogzArgs {
  int32_t problem_type, num_instances, chunk_bits;
  double beta;
  const int32_t* n;
  const int32_t* ld;
  const int64_t* j_off;
  const int64_t* h_off;
  const float* J;
  const float* h;
  double* part_max;  // [num_instances, blocks]
  double* part_sum;
};

// max_samples: the largest reads[b] (bounds the grid).
cudaError_t launch_ais(const AisArgs& a, int64_t max_samples, cudaStream_t st);
// Visiting orders of sweeps 0 .. count-1 of every instance into
// out[(sweep * num_instances + inst) * max_n + i].
cudaError_t launch_perm_all(const int32_t* n_tab, int num_instances, int max_n,
                            int count, uint64_t seed, int32_t* out,
                            cudaStream_t st);
cudaError_t launch_logz(const LogzArgs& a, int max_n, cudaStream_t st);

}  // namespace pysa_gb
