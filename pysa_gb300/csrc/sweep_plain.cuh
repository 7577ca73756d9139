// sweep_plain.cuh -- the plain Metropolis sweep on CUDA cores (sm_103a).
//
// One sweep of pysa/simulation.py:60-76 (sequential) or :41-57 (random order)
// for a block of chains of one instance, using the local-field form of the
// rule in pysa/ising.py:40-63 / pysa/qubo.py:40-63:
//     dn = 2 s_i H_i (Ising) or (2 x_i - 1) H_i (QUBO),  H = J s + h,
// so a decision costs O(1) and only an accepted flip costs O(N):
//     H[c, :] += delta_c * J[i, :].
//
// Layout.  A warp owns GW chains; lane l owns columns l, l+32, ... of each,
// so H[g][m] (register) is the field of chain g at column 32 m + l.  All
// chains of the CTA visit spin i together: row J[i, :] is staged into shared
// memory ONCE per CTA by the TMA engine (cp.async.bulk) through a ring of RB
// rows and read by every warp.  Rows are stored packed so that lane l's NC
// values are contiguous (LDS.128).  The GW decisions of a step run on lanes
// 0..GW-1 in parallel (values moved by warp shuffles), the accept mask is a
// warp ballot, and the rank-1 field update is a warp-uniform loop.
//
// The last warp to finish with a ring slot refills it (shared-memory atomic
// counter + proxy fence + bulk copy), so no warp ever waits for a producer.
#pragma once
#include "common.cuh"

namespace pysa_gb {

template <int NC>
struct PackedRow {
  // floats per lane in a packed row: NC rounded so that lane strides are
  // 16-B aligned and an odd number of 16-B units (conflict-free LDS.128)
  static constexpr int LS = NC < 4 ? 4 : (((NC / 4) & 1) ? NC : NC + 4);
  static constexpr int ROW = 32 * LS;
};

struct SweepItem {
  int32_t inst, chain0, nchains, variant;
  int32_t poff_lo, poff_hi, pad0, pad1;
};

struct PlainArgs {
  pysa_gb_problems p;
  pysa_gb_state s;
  const float* packed_j;
  const int32_t* perm;
  float* fields;
  int32_t field_ld;
  int32_t perm_slots;
  const SweepItem* items;
  int32_t num_items;
  int32_t update;
  uint64_t seed;
  const int32_t* skip_inst;  // [num_instances] 1 = handled elsewhere; or null
};

// Wait bounded by wall time (about one second), then report and give up.
__device__ __forceinline__ bool mbar_wait_timed(uint64_t* bar, uint32_t parity,
                                                int32_t* status) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (globaltimer_ns() - t0 > 1000000000ull) {
      set_status(status, PYSA_GB_ERR_TIMEOUT);
      return false;
    }
  }
}

template <int NC, int GW, int W, int RB>
struct PlainSmem {
  static constexpr int ROW = PackedRow<NC>::ROW;
  static constexpr size_t ring = sizeof(float) * RB * ROW;
  static constexpr size_t bars = sizeof(uint64_t) * RB;
  static constexpr size_t cnts = sizeof(uint32_t) * RB;
  static constexpr size_t perm = sizeof(int32_t) * 32 * NC;
  static constexpr size_t spin = sizeof(uint32_t) * W * NC * GW;
  static constexpr size_t fmir_per_warp = sizeof(float) * GW * (32 * NC + 1);
  static constexpr size_t base = ring + bars + cnts + perm + spin;
  static size_t bytes(bool random) {
    return base + (random ? fmir_per_warp * W : 0);
  }
};

template <int NC, int GW, int W, int RB, bool RANDOM>
__global__ void __launch_bounds__(W * 32, 1)
    k_sweep_plain(const PlainArgs a) {
  using L = PackedRow<NC>;
  using S = PlainSmem<NC, GW, W, RB>;
  extern __shared__ __align__(128) unsigned char smem[];
  float* ring = reinterpret_cast<float*>(smem);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + S::ring);
  uint32_t* cnt = reinterpret_cast<uint32_t*>(smem + S::ring + S::bars);
  int32_t* perm_s =
      reinterpret_cast<int32_t*>(smem + S::ring + S::bars + S::cnts);
  uint32_t* spin_s = reinterpret_cast<uint32_t*>(smem + S::ring + S::bars +
                                                 S::cnts + S::perm);
  float* fmir = reinterpret_cast<float*>(smem + S::base);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool ising = a.p.problem_type == PYSA_GB_ISING;
  int32_t* status = a.s.status;
  const uint32_t sweep = (uint32_t)(*a.s.sweep_counter);

  if (threadIdx.x == 0) {
    for (int r = 0; r < RB; ++r) {
      mbar_init(&full[r], 1);
      cnt[r] = 0;
    }
    fence_mbar_init();
  }
  __syncthreads();

  uint32_t T = 0;  // ring position, continuous across items
  uint32_t* my_spin = spin_s + warp * NC * GW;
  float* my_fmir = fmir + (size_t)warp * GW * (32 * NC + 1);

  for (int it = blockIdx.x; it < a.num_items; it += gridDim.x) {
    const SweepItem item = a.items[it];
    const int inst = item.inst;
    if (a.skip_inst && a.skip_inst[inst]) continue;  // uniform per CTA
    const int n = a.p.n[inst];
    const int words = (n + 31) >> 5;
    const int64_t chain_base = a.p.chain_off[inst];
    const float* Jp =
        a.packed_j + (((int64_t)item.poff_hi << 32) | (uint32_t)item.poff_lo);
    const int32_t* perm_g =
        a.perm + ((int64_t)(sweep % (uint32_t)a.perm_slots) *
                      a.p.num_instances + inst) * (int64_t)a.p.max_n;
    if (RANDOM)
      for (int t = threadIdx.x; t < n; t += blockDim.x) perm_s[t] = perm_g[t];
    __syncthreads();
    if (threadIdx.x == 0) {
      const int first = n < RB ? n : RB;
      for (int r = 0; r < first; ++r) {
        const int slot = (T + r) % RB;
        const int row = RANDOM ? perm_s[r] : r;
        mbar_expect_tx_arrive(&full[slot], L::ROW * 4);
        bulk_g2s(ring + slot * L::ROW, Jp + (int64_t)row * L::ROW,
                 L::ROW * 4, &full[slot]);
      }
    }

    // ---- load this warp's chains
    const int g0 = warp * GW;  // first chain of the warp within the item
    int64_t chain[GW];
    float H[GW][NC];
#pragma unroll
    for (int g = 0; g < GW; ++g) {
      const bool valid = g0 + g < item.nchains;
      chain[g] = item.chain0 + g0 + g;
      const float* f = a.fields + chain[g] * a.field_ld;
#pragma unroll
      for (int m = 0; m < NC; ++m) {
        const int col = 32 * m + lane;
        H[g][m] = (valid && col < n) ? f[col] : 0.0f;
      }
    }
    for (int idx = lane; idx < NC * GW; idx += 32) {
      const int m = idx / GW, g = idx % GW;
      const bool valid = g0 + g < item.nchains && m < words;
      my_spin[idx] =
          valid ? a.s.spins[(item.chain0 + g0 + g) * (int64_t)a.p.words + m] : 0u;
    }
    if (RANDOM) {
#pragma unroll
      for (int g = 0; g < GW; ++g)
#pragma unroll
        for (int m = 0; m < NC; ++m)
          my_fmir[g * (32 * NC + 1) + 32 * m + lane] = H[g][m];
    }
    // lane g (< GW) carries chain g's decision state
    const int gl = lane < GW ? lane : 0;
    const bool lane_valid = lane < GW && g0 + lane < item.nchains;
    const int64_t my_chain = item.chain0 + g0 + gl;
    const float beta = lane_valid ? a.s.chain_beta[my_chain] : 0.0f;
    double dE = 0.0;
    float dE_chunk = 0.0f;
    __syncwarp();

    constexpr int JC = (GW + 3) / 4;  // Philox calls per lane per 32 steps
    uint32_t rnd[JC][4];
    float hc[GW];  // sequential order: field of the current 32-column chunk
    bool abort = false;

    for (int t = 0; t < n; ++t) {
      const uint32_t pos_T = T + t;
      const int slot = pos_T % RB;
      const int i = RANDOM ? perm_s[t] : t;
      const int m = i >> 5, l = i & 31;
      const int p = t & 31;

      if (p == 0) {
        // uniforms for steps t..t+31 of every chain of the warp
#pragma unroll
        for (int j = 0; j < JC; ++j) {
          const int P = j * 32 + lane, g = P >> 3, q = P & 7;
          const int gg = g < GW ? g : 0;
          const uint32_t cl = (uint32_t)(item.chain0 + g0 + gg - chain_base);
          draw4(g0 + gg < item.nchains
                    ? chain_seed(a.seed, a.s.stream_key, item.chain0 + g0 + gg)
                    : a.seed,
                TAG_SWEEP, (uint32_t)inst, sweep, cl,
                (uint32_t)((t >> 2) + q), rnd[j]);
        }
        if (!RANDOM) {
#pragma unroll
          for (int g = 0; g < GW; ++g) {
            float v = H[g][0];
#pragma unroll
            for (int mm = 1; mm < NC; ++mm) v = (mm == m) ? H[g][mm] : v;
            hc[g] = v;
          }
        }
      }

      // field of spin i for lane g's chain
      float hv = 0.0f;
      if (RANDOM) {
        if (lane < GW) hv = my_fmir[lane * (32 * NC + 1) + i];
      } else {
#pragma unroll
        for (int g = 0; g < GW; ++g) {
          const float v = __shfl_sync(0xffffffffu, hc[g], l);
          if (lane == g) hv = v;
        }
      }
      // uniform of step t for lane g's chain
      uint32_t x = 0;
      {
        const int c = p & 3, q = p >> 2;
        const int src = 8 * (lane & 3) + q;
#pragma unroll
        for (int j = 0; j < JC; ++j) {
          const uint32_t r = c == 0 ? rnd[j][0]
                             : c == 1 ? rnd[j][1]
                             : c == 2 ? rnd[j][2]
                                      : rnd[j][3];
          const uint32_t v = __shfl_sync(0xffffffffu, r, src);
          if ((lane >> 2) == j) x = v;
        }
      }
      const uint32_t word = my_spin[m * GW + gl];
      const bool sbit = (word >> l) & 1u;
      const float dn = ising ? (sbit ? 2.0f * hv : -2.0f * hv)
                             : (sbit ? hv : -hv);
      const bool acc = lane_valid && metropolis_accept(dn, beta, x);
      const uint32_t am = __ballot_sync(0xffffffffu, acc);
      const uint32_t sm = __ballot_sync(0xffffffffu, sbit);
      if (acc) {
        my_spin[m * GW + gl] = word ^ (1u << l);
        dE_chunk -= dn;
      }

      // wait for row i in the ring, then apply the accepted flips
      if (!mbar_wait_timed(&full[slot], (pos_T / RB) & 1u, status)) {
        abort = true;
        break;
      }
      if (am) {
        const float* row = ring + slot * PackedRow<NC>::ROW + lane * L::LS;
        const float Jc = row[m];
        if constexpr (GW == 1) {
          // one chain: stream the row straight into the FMAs
          const float d = ising ? ((sm & 1u) ? -2.0f : 2.0f)
                                : ((sm & 1u) ? -1.0f : 1.0f);
#pragma unroll
          for (int k = 0; k < L::LS / 4; ++k) {
            const float4 v = reinterpret_cast<const float4*>(row)[k];
            if (4 * k + 0 < NC) H[0][4 * k + 0] = fmaf(d, v.x, H[0][4 * k + 0]);
            if (4 * k + 1 < NC) H[0][4 * k + 1] = fmaf(d, v.y, H[0][4 * k + 1]);
            if (4 * k + 2 < NC) H[0][4 * k + 2] = fmaf(d, v.z, H[0][4 * k + 2]);
            if (4 * k + 3 < NC) H[0][4 * k + 3] = fmaf(d, v.w, H[0][4 * k + 3]);
          }
          if (RANDOM) {
#pragma unroll
            for (int mm = 0; mm < NC; ++mm)
              my_fmir[32 * mm + lane] = H[0][mm];
          } else {
            hc[0] = fmaf(d, Jc, hc[0]);
          }
        } else {
          float Jr[NC];
#pragma unroll
          for (int k = 0; k < L::LS / 4; ++k) {
            const float4 v = reinterpret_cast<const float4*>(row)[k];
            if (4 * k + 0 < NC) Jr[4 * k + 0] = v.x;
            if (4 * k + 1 < NC) Jr[4 * k + 1] = v.y;
            if (4 * k + 2 < NC) Jr[4 * k + 2] = v.z;
            if (4 * k + 3 < NC) Jr[4 * k + 3] = v.w;
          }
#pragma unroll
          for (int g = 0; g < GW; ++g) {
            if ((am >> g) & 1u) {
              const bool sg = (sm >> g) & 1u;
              const float d =
                  ising ? (sg ? -2.0f : 2.0f) : (sg ? -1.0f : 1.0f);
#pragma unroll
              for (int mm = 0; mm < NC; ++mm)
                H[g][mm] = fmaf(d, Jr[mm], H[g][mm]);
              if (RANDOM) {
#pragma unroll
                for (int mm = 0; mm < NC; ++mm)
                  my_fmir[g * (32 * NC + 1) + 32 * mm + lane] = H[g][mm];
              } else {
                hc[g] = fmaf(d, Jc, hc[g]);
              }
            }
          }
        }
      }
      __syncwarp();
      // release the slot; the last warp refills it with the row of step t+RB
      if (lane == 0) {
        __threadfence_block();
        const uint32_t old = atomicAdd(&cnt[slot], 1u);
        if (old == W - 1) {
          cnt[slot] = 0;
          if (t + RB < n) {
            const int row = RANDOM ? perm_s[t + RB] : t + RB;
            fence_proxy_async();
            mbar_expect_tx_arrive(&full[slot], L::ROW * 4);
            bulk_g2s(ring + slot * L::ROW, Jp + (int64_t)row * L::ROW,
                     L::ROW * 4, &full[slot]);
          }
        }
      }
      if (p == 31 || t == n - 1) {
        dE += (double)dE_chunk;
        dE_chunk = 0.0f;
      }
    }
    if (abort) return;
    T += n;

    // ---- write back fields, spins, energies; track the best state
#pragma unroll
    for (int g = 0; g < GW; ++g) {
      if (g0 + g < item.nchains) {
        float* f = a.fields + chain[g] * a.field_ld;
#pragma unroll
        for (int m = 0; m < NC; ++m) {
          const int col = 32 * m + lane;
          if (col < n) f[col] = H[g][m];
        }
      }
    }
    __syncwarp();
    float e_new = 0.0f;
    bool improved = false;
    if (lane_valid) {
      e_new = (float)((double)a.s.energies[my_chain] + dE);
      a.s.energies[my_chain] = e_new;
      if (e_new < a.s.best_energy[my_chain]) {
        improved = true;
        a.s.best_energy[my_chain] = e_new;
        a.s.best_sweep[my_chain] = (int32_t)sweep;
      }
    }
    const uint32_t imp = __ballot_sync(0xffffffffu, improved);
#pragma unroll
    for (int g = 0; g < GW; ++g) {
      if (g0 + g < item.nchains) {
        const int64_t c = item.chain0 + g0 + g;
        for (int w = lane; w < words; w += 32) {
          const uint32_t v = my_spin[w * GW + g];
          a.s.spins[c * a.p.words + w] = v;
          if ((imp >> g) & 1u) a.s.best_spins[c * a.p.words + w] = v;
        }
      }
    }
    __syncthreads();  // ring and perm reuse by the next item
  }
}

}  // namespace pysa_gb
