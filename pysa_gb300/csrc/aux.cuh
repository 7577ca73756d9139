// aux.cuh -- argument blocks and launchers of the kernels around the sweep.
#pragma once
#include "common.cuh"

namespace pysa_gb {

// Largest R the exchange kernel stages in shared memory.
constexpr int kMaxReplicas = 512;

struct PrepArgs {
  pysa_gb_problems p;
  pysa_gb_state s;
  float* fields;
  int32_t field_ld;
  int32_t set_energies;
  int32_t init_best;
  int32_t best_global;
};

struct XArgs {
  pysa_gb_problems p;
  pysa_gb_state s;
  uint64_t seed;
  int32_t use_pt;
  int32_t log_omega_stride;
  int32_t exchange_every;  // <= 1: every sweep; k: after sweeps (s+1) % k == 0
  int32_t pad_;
};

// Whether sweep `sweep` ends with a replica exchange.
__host__ __device__ inline bool exchange_after(int32_t every, uint32_t sweep) {
  return every <= 1 || (sweep + 1u) % (uint32_t)every == 0u;
}

struct PermArgs {
  pysa_gb_problems p;
  const int64_t* sweep_counter;
  int32_t* perm;
  int32_t perm_slots;
  uint64_t seed;
};

void launch_pack_rows(const float* J, int ld, int n, int nc, int ls,
                      float* packed, cudaStream_t st);
void launch_prepare(const PrepArgs& a, cudaStream_t st);
void launch_exchange(const XArgs& a, cudaStream_t st);
// Visiting orders of the current sweep and the count - 1 after it (slots
// sweep % perm_slots).
void launch_perm(const PermArgs& a, cudaStream_t st, int count = 1);
void launch_energy64(int ptype, int n, int ld, const double* J,
                     const double* h, const uint32_t* spins, int words,
                     int64_t count, double* out, cudaStream_t st);
void launch_energy64_tables(const pysa_gb_problems& p, int inst,
                            const uint32_t* spins, int words, int64_t count,
                            double* out, cudaStream_t st);
void launch_unpack(int ptype, int n, const uint32_t* spins, int words,
                   int64_t count, float* out, int out_ld, cudaStream_t st);
void launch_pack(int ptype, int n, const float* x, int x_ld, int64_t count,
                 uint32_t* spins, int words, cudaStream_t st);
void launch_load_problem(const pysa_gb_problems& p, int inst, int n, int ld,
                         const float* P, int p_ld, cudaStream_t st);

}  // namespace pysa_gb
