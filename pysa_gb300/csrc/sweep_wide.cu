// sweep_wide.cu -- the plain Metropolis sweep for dense instances too wide
// for the register-resident kernel (n > 4096 spins).
//
// Same sweep as pysa/simulation.py:60-76 (sequential) or :41-57 (random
// order) with the rule of pysa/ising.py:40-63 / pysa/qubo.py:40-63 in the
// local-field form (dn from the field H_i of the spin; an accepted flip adds
// delta * J[i, :] to H), as the register-resident plain kernel does, but the
// fields of a chain live in global memory (L2-resident: n floats per chain)
// instead of registers, so any n works.
//
// One warp per chain, kWideWarps chains per CTA.  The visiting positions of
// the next 32 steps are handled in chunks: lane l holds the field of the
// chunk's position l in a register (loaded once per chunk and corrected on
// every accepted flip of the chunk), so a decision is two warp shuffles and
// no memory access; an accepted flip streams the chain's field row against
// row i of J (float4, coalesced) and corrects the chunk's registers.  The
// chain's spin words sit in shared memory.  Decisions are made by every lane
// on the same values, so the flip branch is warp-uniform.  Uniforms come
// from the sweep stream exactly as in the other sweep kernels.
#include "common.cuh"
#include "sweep_plain.cuh"
#include "wide_api.h"

namespace pysa_gb {

template <bool RANDOM>
__global__ void __launch_bounds__(32 * kWideWarps)
    k_sweep_wide(const WideArgs a) {
  extern __shared__ uint32_t spin_s[];  // [kWideWarps][a.p.words]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool ising = a.p.problem_type == PYSA_GB_ISING;
  const uint32_t sweep = (uint32_t)(*a.s.sweep_counter);
  uint32_t* sp = spin_s + (size_t)warp * a.p.words;

  for (int it = blockIdx.x; it < a.num_items; it += gridDim.x) {
    const SweepItem item = a.items[it];
    if (warp >= item.nchains) continue;  // warps are independent
    const int inst = item.inst;
    const int n = a.p.n[inst], ld = a.p.ld[inst];
    const int words = (n + 31) >> 5;
    const int64_t chain = item.chain0 + warp;
    const uint32_t cl = (uint32_t)(chain - a.p.chain_off[inst]);
    const float* J = a.p.J + a.p.j_off[inst];
    float* H = a.fields + chain * (int64_t)a.field_ld;
    const int32_t* perm =
        a.perm + ((int64_t)(sweep % (uint32_t)a.perm_slots) *
                      a.p.num_instances + inst) * (int64_t)a.p.max_n;
    const uint64_t seed = chain_seed(a.seed, a.s.stream_key, chain);
    const float beta = a.s.chain_beta[chain];
    for (int w = lane; w < words; w += 32)
      sp[w] = a.s.spins[chain * (int64_t)a.p.words + w];
    __syncwarp();

    double dE = 0.0;
    for (int t0 = 0; t0 < n; t0 += 32) {
      // the chunk: position t0 + lane, its spin, field and uniform
      const int tl = t0 + lane;
      const int il = tl < n ? (RANDOM ? perm[tl] : tl) : -1;
      float hc = il >= 0 ? H[il] : 0.0f;
      uint32_t r4[4];
      draw4(seed, TAG_SWEEP, (uint32_t)inst, sweep, cl, (uint32_t)(tl >> 2),
            r4);
      const uint32_t q = (uint32_t)tl & 3u;
      const uint32_t xl = q == 0 ? r4[0] : q == 1 ? r4[1] : q == 2 ? r4[2]
                                                                   : r4[3];
      const int kend = n - t0 < 32 ? n - t0 : 32;
      float dEc = 0.0f;
      for (int k = 0; k < kend; ++k) {
        const int i = __shfl_sync(0xffffffffu, il, k);
        const float h = __shfl_sync(0xffffffffu, hc, k);
        const uint32_t x = __shfl_sync(0xffffffffu, xl, k);
        const bool s = (sp[i >> 5] >> (i & 31)) & 1u;
        const float dn = ising ? (s ? 2.0f * h : -2.0f * h) : (s ? h : -h);
        if (!metropolis_accept(dn, beta, x)) continue;  // warp-uniform
        dEc -= dn;
        const float d = ising ? (s ? -2.0f : 2.0f) : (s ? -1.0f : 1.0f);
        const float* Jr = J + (int64_t)i * ld;
        // H += d * J[i, :]: float4 over the columns, scalar tail
        const int n4 = n & ~3;
        for (int c = 4 * lane; c < n4; c += 128) {
          const float4 jv = __ldg(reinterpret_cast<const float4*>(Jr + c));
          float4 hv = *reinterpret_cast<float4*>(H + c);
          hv.x = fmaf(d, jv.x, hv.x);
          hv.y = fmaf(d, jv.y, hv.y);
          hv.z = fmaf(d, jv.z, hv.z);
          hv.w = fmaf(d, jv.w, hv.w);
          *reinterpret_cast<float4*>(H + c) = hv;
        }
        if (n4 + lane < n) H[n4 + lane] = fmaf(d, __ldg(Jr + n4 + lane),
                                               H[n4 + lane]);
        if (il >= 0) hc = fmaf(d, __ldg(Jr + il), hc);
        if (lane == 0) sp[i >> 5] ^= 1u << (i & 31);
        __syncwarp();  // field row and spin word seen by every lane
      }
      dE += (double)dEc;
    }

    // spins, energy and best state back to the chain
    for (int w = lane; w < words; w += 32)
      a.s.spins[chain * (int64_t)a.p.words + w] = sp[w];
    bool improved = false;
    if (lane == 0) {
      const float e = (float)((double)a.s.energies[chain] + dE);
      a.s.energies[chain] = e;
      if (e < a.s.best_energy[chain]) {
        improved = true;
        a.s.best_energy[chain] = e;
        a.s.best_sweep[chain] = (int32_t)sweep;
      }
    }
    if (__shfl_sync(0xffffffffu, improved, 0))
      for (int w = lane; w < words; w += 32)
        a.s.best_spins[chain * (int64_t)a.p.words + w] = sp[w];
    __syncwarp();  // spin words reused by this warp's next item
  }
}

size_t wide_smem_bytes(int words) {
  return sizeof(uint32_t) * (size_t)kWideWarps * (size_t)words;
}

cudaError_t launch_wide(const WideArgs& a, bool random, int max_ctas,
                        cudaStream_t st) {
  if (a.num_items <= 0) return cudaSuccess;
  const size_t sm = wide_smem_bytes(a.p.words);
  const void* f = random ? (const void*)k_sweep_wide<true>
                         : (const void*)k_sweep_wide<false>;
  if (sm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(
        f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  const int grid = a.num_items < max_ctas ? a.num_items : max_ctas;
  if (random)
    k_sweep_wide<true><<<grid, 32 * kWideWarps, sm, st>>>(a);
  else
    k_sweep_wide<false><<<grid, 32 * kWideWarps, sm, st>>>(a);
  return cudaGetLastError();
}

}  // namespace pysa_gb
