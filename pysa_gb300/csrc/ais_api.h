// ais_api.h -- argument blocks of the AIS and exact log-Z kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pysa_gb {

struct AisArgs {
  int32_t problem_type, n, ld, words, num_temps, update, ref, order, inst,
      max_n;
  int64_t samples;
  double p;
  uint64_t seed;
  const float* J;        // transposed couplings (row i = field change of i)
  const float* temps;    // [num_temps] anneal schedule
  const int32_t* perm;   // [num_temps, max_n] visiting orders (random)
  const float* fields;   // [samples, field_ld] initial local fields
  int32_t field_ld;
  uint32_t* spins;       // [samples, words] in/out
  float* energies;       // [samples] in/out
  double* log_w;         // [samples] out
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

cudaError_t launch_ais(const AisArgs& a, cudaStream_t st);
cudaError_t launch_perm_range(int n, int max_n, uint32_t inst, uint32_t first,
                              int count, uint64_t seed, int32_t* out,
                              cudaStream_t st);
cudaError_t launch_logz(const LogzArgs& a, int max_n, cudaStream_t st);

}  // namespace pysa_gb
