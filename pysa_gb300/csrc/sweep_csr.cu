// sweep_csr.cu -- the Metropolis sweep for sparse couplings on CUDA cores
// (sm_103a).
//
// Same sweep as pysa/simulation.py:60-76 (sequential) / :41-57 (random
// order) with the rule of pysa/ising.py:40-63 / pysa/qubo.py:40-63, but the
// field of spin i is recomputed from the nonzero couplings of row i instead
// of a dense dot, so an attempt costs O(degree).  One thread per chain; the
// CTA's 128 chains keep their spins bit-packed in shared memory ([word]
// [chain], so the threads' words are consecutive); all of them visit spin i
// together, so the row's entries are the same addresses for every thread
// (broadcast loads through L1).
//
// Row layout: the entries of row i are grouped by column % 8 (ascending
// column inside a group) and rows[9 i + k] .. rows[9 i + k + 1] delimit group
// k; or, when every row has at most 32 entries, each row is a fixed record
// of D = 4, 8, 16 or 32 entries in that order (bit 31 of the column marks
// the last entry of a group, padding entries have value 0), read with
// vector loads all at once.  The field is summed as eight partial sums, one per group, added in
// group order, then h_i: the fixed-order f32 dot of the oracle with its zero
// terms left out (adding a zero product changes no partial sum), so
// trajectories equal the oracle's for any couplings, not only integer ones.
#include "common.cuh"
#include "csr_api.h"
#include "sweep_plain.cuh"

namespace pysa_gb {

// Asynchronous global -> shared copies (no register staging).
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                   smem_addr(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                   smem_addr(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// Fixed records are staged 32 visiting positions at a time into a double
// buffer of shared memory, one row per thread of the first warp, while the
// previous 32 are decided: [D columns][D values][h_i][pad] per row.
template <int D>
struct RecSlab {
  static constexpr int STRIDE = 2 * D + 4;  // floats per staged row
  static constexpr size_t BYTES = D > 0 ? (size_t)2 * 32 * STRIDE * 4 : 0;
};

// One staged fixed record in registers (all lanes read the same row of the
// slab: broadcast loads).
template <int D>
struct Rec {
  int32_t cols[D];
  float vals[D];
  float h;
  __device__ __forceinline__ void load(const float* rec) {
#pragma unroll
    for (int q = 0; q < D / 4; ++q) {
      const int4 c4 = reinterpret_cast<const int4*>(rec)[q];
      const float4 v4 = reinterpret_cast<const float4*>(rec + D)[q];
      cols[4 * q + 0] = c4.x; cols[4 * q + 1] = c4.y;
      cols[4 * q + 2] = c4.z; cols[4 * q + 3] = c4.w;
      vals[4 * q + 0] = v4.x; vals[4 * q + 1] = v4.y;
      vals[4 * q + 2] = v4.z; vals[4 * q + 3] = v4.w;
    }
    h = rec[2 * D];
  }
  // field sum over the current spins; a group's partial sum joins the
  // total at the entry flagged last in it
  __device__ __forceinline__ float dot(const uint32_t* my, int CH,
                                       bool ising) const {
    uint32_t words[D];
#pragma unroll
    for (int e = 0; e < D; ++e) {
      const int c = cols[e] & 0x7fffffff;
      words[e] = my[(c >> 5) * CH];
    }
    float sum = 0.0f, part = 0.0f;
#pragma unroll
    for (int e = 0; e < D; ++e) {
      const int c = cols[e] & 0x7fffffff;
      const bool bit = (words[e] >> (c & 31)) & 1u;
      if (ising)
        part += bit ? vals[e] : -vals[e];
      else if (bit)
        part += vals[e];
      if (cols[e] < 0) {  // last entry of its group
        sum += part;
        part = 0.0f;
      }
    }
    return sum;
  }
};

template <bool RANDOM, int D>
__global__ void __launch_bounds__(kCsrChains) k_sweep_csr(const CsrArgs a) {
  const int CH = blockDim.x;  // chains per CTA = the spin words' stride
  extern __shared__ __align__(16) uint32_t smem_u[];
  const SweepItem item = a.items[blockIdx.x];
  const int inst = item.inst;
  const int n = a.p.n[inst];
  const int words = (n + 31) >> 5;
  uint32_t* spin_s = smem_u;  // [words][CH]
  float* slab = reinterpret_cast<float*>(smem_u + words * CH);  // RecSlab<D>
  int32_t* perm_s =
      reinterpret_cast<int32_t*>(smem_u + words * CH + RecSlab<D>::BYTES / 4);
  __shared__ uint8_t imp_s[kCsrChains];
  const int tid = threadIdx.x;
  const bool valid = tid < item.nchains;
  const int64_t chain = item.chain0 + tid;
  const bool ising = a.p.problem_type == PYSA_GB_ISING;
  const uint32_t sweep = (uint32_t)(*a.s.sweep_counter);

  // spins in, coalesced over (chain, word)
  for (int idx = tid; idx < CH * words; idx += blockDim.x) {
    const int c = idx / words, w = idx - c * words;
    spin_s[w * CH + c] =
        c < item.nchains
            ? a.s.spins[(item.chain0 + c) * (int64_t)a.p.words + w]
            : 0u;
  }
  if (RANDOM) {
    const int32_t* perm_g =
        a.perm + ((int64_t)(sweep % (uint32_t)a.perm_slots) *
                      a.p.num_instances + inst) * (int64_t)a.p.max_n;
    for (int t = tid; t < n; t += blockDim.x) perm_s[t] = perm_g[t];
  }
  __syncthreads();

  const float beta = valid ? a.s.chain_beta[chain] : 0.0f;
  const uint32_t cl = (uint32_t)(chain - a.p.chain_off[inst]);
  const uint64_t seed_c =
      valid ? chain_seed(a.seed, a.s.stream_key, chain) : a.seed;
  const int32_t* rows =
      D > 0 ? nullptr : a.p.csr_rows + a.p.csr_row_off[inst] * 9;
  const int32_t* colp = a.p.csr_col + a.p.csr_ent_off[inst];
  const float* valp = a.p.csr_val + a.p.csr_ent_off[inst];
  const float* h = a.p.h + a.p.h_off[inst];
  uint32_t* my = spin_s + tid;
  double dE = 0.0;

  // rows of visiting positions 32 b .. 32 b + 31 into slab buffer b & 1
  auto stage = [&](int b) {
    if constexpr (D > 0) {
      const int t = 32 * b + tid;
      if (tid < 32 && t < n) {
        const int i = RANDOM ? perm_s[t] : t;
        float* dst = slab + ((b & 1) * 32 + tid) * RecSlab<D>::STRIDE;
#pragma unroll
        for (int q = 0; q < D / 4; ++q) {
          cp_async16(dst + 4 * q, colp + (int64_t)i * D + 4 * q);
          cp_async16(dst + D + 4 * q, valp + (int64_t)i * D + 4 * q);
        }
        cp_async4(dst + 2 * D, h + i);
      }
      cp_async_commit();
    }
  };
  stage(0);
  if constexpr (D > 0) {
    cp_async_wait_all();
    __syncthreads();
  }
  const int nb = (n + 31) >> 5;
  for (int b = 0; b < nb; ++b) {
    if (b + 1 < nb) stage(b + 1);
    for (int t0 = 32 * b; t0 < n && t0 < 32 * b + 32; t0 += 4) {
      uint32_t rnd[4];
      draw4(seed_c, TAG_SWEEP, (uint32_t)inst, sweep, cl,
            (uint32_t)(t0 >> 2), rnd);
      // short records: all four up front, ahead of the flips' shared
      // stores; long ones one at a time (registers)
      constexpr bool kHoist = D > 0 && D <= 8;
      Rec<(D > 0 ? D : 4)> recs[kHoist ? 4 : 1];
      if constexpr (kHoist) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          recs[q].load(slab + ((b & 1) * 32 + ((t0 + q) & 31)) *
                                  RecSlab<D>::STRIDE);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int t = t0 + q;
        if (t >= n) break;
        const int i = RANDOM ? perm_s[t] : t;
        float sum = 0.0f, hi;
        if constexpr (D > 0) {
          auto& r = recs[kHoist ? q : 0];
          if constexpr (!kHoist)
            r.load(slab + ((b & 1) * 32 + (t & 31)) * RecSlab<D>::STRIDE);
          sum = r.dot(my, CH, ising);
          hi = r.h;
        } else {
          const int32_t* r9 = rows + (int64_t)i * 9;
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            float part = 0.0f;
            const int e1 = __ldg(r9 + k + 1);
            for (int e = __ldg(r9 + k); e < e1; ++e) {
              const int col = __ldg(colp + e);
              const float v = __ldg(valp + e);
              const bool bit = (my[(col >> 5) * CH] >> (col & 31)) & 1u;
              if (ising)
                part += bit ? v : -v;
              else if (bit)
                part += v;
            }
            sum += part;
          }
          hi = __ldg(h + i);
        }
        const float field = sum + hi;
        const uint32_t wi = my[(i >> 5) * CH];
        const bool sbit = (wi >> (i & 31)) & 1u;
        const float dn = ising ? (sbit ? 2.0f * field : -2.0f * field)
                               : (sbit ? field : -field);
        if (valid && metropolis_accept(dn, beta, rnd[q])) {
          my[(i >> 5) * CH] = wi ^ (1u << (i & 31));
          dE -= (double)dn;  // the sweep's energy change, summed in f64
        }
      }
    }
    if constexpr (D > 0) {
      cp_async_wait_all();
      __syncthreads();  // buffer b & 1 free, b + 1 landed
    }
  }

  // energies and the per-chain best (strict <, pysa/simulation.py:150-171)
  bool improved = false;
  if (valid) {
    const float e_new = (float)((double)a.s.energies[chain] + dE);
    a.s.energies[chain] = e_new;
    if (e_new < a.s.best_energy[chain]) {
      improved = true;
      a.s.best_energy[chain] = e_new;
      a.s.best_sweep[chain] = (int32_t)sweep;
    }
  }
  imp_s[tid] = improved ? 1 : 0;
  __syncthreads();
  for (int idx = tid; idx < item.nchains * words; idx += blockDim.x) {
    const int c = idx / words, w = idx - c * words;
    const uint32_t v = spin_s[w * CH + c];
    const int64_t off = (item.chain0 + c) * (int64_t)a.p.words + w;
    a.s.spins[off] = v;
    if (imp_s[c]) a.s.best_spins[off] = v;
  }
}

template <bool RANDOM, int D>
static cudaError_t launch_csr_t(const CsrArgs& a, size_t base,
                                cudaStream_t st) {
  const size_t smem = base + RecSlab<D>::BYTES;
  cudaError_t e = cudaFuncSetAttribute(
      k_sweep_csr<RANDOM, D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)smem);
  if (e != cudaSuccess) return e;
  k_sweep_csr<RANDOM, D><<<a.num_items, a.chains, smem, st>>>(a);
  return cudaGetLastError();
}

template <bool RANDOM>
static cudaError_t launch_csr_w(const CsrArgs& a, size_t smem,
                                cudaStream_t st) {
  switch (a.width) {
    case 4: return launch_csr_t<RANDOM, 4>(a, smem, st);
    case 8: return launch_csr_t<RANDOM, 8>(a, smem, st);
    case 16: return launch_csr_t<RANDOM, 16>(a, smem, st);
    case 32: return launch_csr_t<RANDOM, 32>(a, smem, st);
    default: return launch_csr_t<RANDOM, 0>(a, smem, st);
  }
}

cudaError_t launch_csr(const CsrArgs& a, bool random, cudaStream_t st) {
  if (a.num_items <= 0) return cudaSuccess;
  const int words = (a.p.max_n + 31) / 32;
  const size_t base = (size_t)words * a.chains * 4 +
                      (random ? (size_t)a.p.max_n * 4 : 0);
  return random ? launch_csr_w<true>(a, base, st)
                : launch_csr_w<false>(a, base, st);
}

}  // namespace pysa_gb
