// ais.cu -- annealed importance sampling and exact log Z (sm_103a).
//
// k_ais restates ais_sample (pysa/simulation.py:293-317) with the acceptance
// rule of update_spin_ref (pysa/ising.py:66-92, pysa/qubo.py:66-92):
//   full = beta dn + (1 - beta) log(p0(s') / p0(s)),  accept iff full >= 0
//   or log(u) < full.  The uniform reference gives a zero log ratio; the
// Bernoulli reference (pysa/ais.py:198-217) gives +-log((1 - p) / p) when a
// bit goes up / down.  Layout as in the plain sweep (warp = GW samples,
// lanes over columns, local fields in registers) but every sample runs its
// whole anneal inside one launch: samples never interact.  The log weight of
// each anneal step is accumulated in f64 (pysa/simulation.py:312-314), after
// the sweep ("reference" order) or before it ("standard" order).
//
// k_logz_exact enumerates all 2^n states in Gray-code order in f64, with an
// online log-sum-exp per thread.
#include "aux.cuh"
#include "ais_api.h"

namespace pysa_gb {

// accept_full on full = beta dn + (1 - beta) refd.  With the uniform
// reference (refd = 0) full = beta dn is exact in f64 and its f32 rounding
// is the f32 product, so the fast path runs on the FP32 pipe (far faster
// than this GPU's FP64 one) and f64 is left to the band's exact rule; the
// decisions are accept_full's.
__device__ __forceinline__ bool ais_accept(float beta, float dn, bool sbit,
                                           double lr, bool uniform_ref,
                                           uint32_t x) {
  if (!uniform_ref) {
    const double refd = sbit ? -lr : lr;  // bit going down : up
    return accept_full(
        (double)beta * (double)dn + (1.0 - (double)beta) * refd, x);
  }
  if (dn != dn) return false;  // as accept_full on a NaN
  // full >= 0: a zero factor or factors of one sign
  if (dn == 0.0f || beta == 0.0f || ((dn > 0.0f) == (beta > 0.0f)))
    return true;
  const float ff = beta * dn;  // == (float)full
  if (ff < -24.0f) return false;
  const float uf = __uint2float_rn(x) * 0x1p-32f + 0x1p-33f;
  const float lf = __logf(uf);
  const float margin = 3e-5f + 1e-6f * fabsf(ff);
  if (lf < ff - margin) return true;
  if (lf > ff + margin) return false;
  return accept_full_slow((double)beta * (double)dn, x);
}

// Log-weight increment of one temperature step,
// (-beta e - (1 - beta) re) - (-beta_old e - (1 - beta_old) re), re the
// reference's log-probability of the state; with the uniform reference
// re = 0 and only the two f32-rounded products remain (same value)
__device__ __forceinline__ double ais_dlw(float beta, float beta_old, float e,
                                         int n, int ones, double logp,
                                         double log1p_, bool uniform_ref) {
  if (uniform_ref)
    return (double)__fmul_rn(-beta, e) - (double)__fmul_rn(-beta_old, e);
  const double re = -((double)(n - ones) * logp + (double)ones * log1p_);
  return ((double)__fmul_rn(-beta, e) - (1.0 - (double)beta) * re) -
         ((double)__fmul_rn(-beta_old, e) - (1.0 - (double)beta_old) * re);
}

template <int NC, int GW>
__global__ void __launch_bounds__(128) k_ais(const AisArgs a) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int inst = blockIdx.y;
  if (a.replicas[inst] != 1) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_status(a.status, PYSA_GB_ERR_ARG);
    return;
  }
  const int n = a.n_tab[inst];
  const int ld = a.ld_tab[inst];
  const int64_t samples = a.reads[inst];
  const int64_t cbase = a.chain_off[inst];
  const float* Jp = a.J + a.j_off[inst];
  const int64_t s0 = (int64_t)warp * GW;
  if (s0 >= samples) return;
  const bool ising = a.problem_type == PYSA_GB_ISING;
  const int words = (n + 31) >> 5;

  float H[GW][NC];
  uint32_t spin[GW][NC];  // word m = spins 32m..32m+31 (same in every lane)
#pragma unroll
  for (int g = 0; g < GW; ++g) {
    const int64_t smp = s0 + g;
    const bool valid = smp < samples;
#pragma unroll
    for (int m = 0; m < NC; ++m) {
      const int col = 32 * m + lane;
      H[g][m] = (valid && col < n)
                    ? a.fields[(cbase + smp) * a.field_ld + col] : 0.0f;
      spin[g][m] =
          (valid && m < words) ? a.spins[(cbase + smp) * a.words + m] : 0u;
    }
  }
  const int gl = lane < GW ? lane : 0;
  const bool lane_valid = lane < GW && s0 + lane < samples;
  const int64_t my = s0 + gl;         // sample index within the instance
  const int64_t myc = cbase + my;     // its chain
  double E = lane_valid ? (double)a.energies[myc] : 0.0;
  int ones = 0;  // bits at 1 (spin +1 / x = 1) of lane g's sample
  if (lane_valid)
    for (int w = 0; w < words; ++w) ones += __popc(a.spins[myc * a.words + w]);
  double lw = 0.0;
  float beta_old = 0.0f;
  const double lr = a.ref == 1 ? log((1.0 - a.p) / a.p) : 0.0;
  const double logp = a.ref == 1 ? log(a.p) : 0.0;
  const double log1p_ = a.ref == 1 ? log(1.0 - a.p) : 0.0;

  for (int k = 0; k < a.num_temps; ++k) {
    const float beta = a.temps[k];
    if (a.order == 1) {
      lw += ais_dlw(beta, beta_old, (float)E, n, ones, logp, log1p_,
                    a.ref != 1);
    }
    const int32_t* perm =
        a.perm + ((int64_t)k * a.num_instances + inst) * a.max_n;
    for (int t = 0; t < n; ++t) {
      const int i = a.update == PYSA_GB_RANDOM ? perm[t] : t;
      const int m = i >> 5, l = i & 31;
      float hv = 0.0f;
      uint32_t word = 0;
#pragma unroll
      for (int g = 0; g < GW; ++g) {
        float hm = H[g][0];
        uint32_t wm = spin[g][0];
#pragma unroll
        for (int mm = 1; mm < NC; ++mm) {
          hm = (mm == m) ? H[g][mm] : hm;
          wm = (mm == m) ? spin[g][mm] : wm;
        }
        const float v = __shfl_sync(0xffffffffu, hm, l);
        if (lane == g) {
          hv = v;
          word = wm;
        }
      }
      const bool sbit = (word >> l) & 1u;
      const float dn = ising ? (sbit ? 2.0f * hv : -2.0f * hv)
                             : (sbit ? hv : -hv);
      bool acc = false;
      if (lane_valid) {
        const uint32_t x = draw1(a.seed, TAG_AIS, (uint32_t)inst, (uint32_t)k,
                                 (uint32_t)my, (uint32_t)t);
        acc = ais_accept(beta, dn, sbit, lr, a.ref != 1, x);
      }
      const uint32_t am = __ballot_sync(0xffffffffu, acc);
      const uint32_t sm = __ballot_sync(0xffffffffu, sbit);
      if (acc) {
        E -= (double)dn;
        ones += sbit ? -1 : 1;
      }
      if (am) {
        const float* row = Jp + (int64_t)i * ld;
        float Jr[NC];
#pragma unroll
        for (int mm = 0; mm < NC; ++mm) {
          const int col = 32 * mm + lane;
          Jr[mm] = col < n ? __ldg(row + col) : 0.0f;
        }
#pragma unroll
        for (int g = 0; g < GW; ++g) {
          if ((am >> g) & 1u) {
            const bool sg = (sm >> g) & 1u;
            const float d = ising ? (sg ? -2.0f : 2.0f) : (sg ? -1.0f : 1.0f);
#pragma unroll
            for (int mm = 0; mm < NC; ++mm) {
              H[g][mm] = fmaf(d, Jr[mm], H[g][mm]);
              if (mm == m) spin[g][mm] ^= (1u << l);
            }
          }
        }
      }
    }
    if (a.order == 0) {
      lw += ais_dlw(beta, beta_old, (float)E, n, ones, logp, log1p_,
                    a.ref != 1);
    }
    beta_old = beta;
  }
  if (lane_valid) {
    a.log_w[myc] = lw;
    a.energies[myc] = (float)E;
  }
#pragma unroll
  for (int g = 0; g < GW; ++g) {
    const int64_t smp = s0 + g;
    if (smp < samples) {
#pragma unroll
      for (int m = 0; m < NC; ++m)
        if (m < words && lane == 0)
          a.spins[(cbase + smp) * a.words + m] = spin[g][m];
    }
  }
}

// Small instances (n <= 32): one thread per sample, its spins in one word
// and its fields in a shared-memory column [32][128] (conflict-free), the
// instance's couplings in shared memory too (the row of the visited spin is
// the same for every thread: a broadcast).  The arithmetic is k_ais's: the
// same f32 field updates (a rejected attempt adds 0 * J, which changes no
// field but possibly the sign of a zero), the same f64 energy and weights,
// the same uniforms (one draw of 4 per 4 steps instead of one per step).
// No shuffles or ballots, and a warp covers 32 samples instead of 8.
__global__ void __launch_bounds__(128) k_ais_small(const AisArgs a) {
  __shared__ float Js[32 * 32];
  __shared__ float Hs[32 * 128];
  const int inst = blockIdx.y;
  const int tid = threadIdx.x;
  if (a.replicas[inst] != 1) {
    if (blockIdx.x == 0 && tid == 0) set_status(a.status, PYSA_GB_ERR_ARG);
    return;
  }
  const int n = a.n_tab[inst];
  const int ld = a.ld_tab[inst];
  const int64_t samples = a.reads[inst];
  if ((int64_t)blockIdx.x * blockDim.x >= samples) return;  // whole CTA
  const float* Jp = a.J + a.j_off[inst];
  for (int e = tid; e < 32 * 32; e += blockDim.x) {
    const int r = e >> 5, c = e & 31;
    Js[e] = (r < n && c < n) ? Jp[(int64_t)r * ld + c] : 0.0f;
  }
  const int64_t my = (int64_t)blockIdx.x * blockDim.x + tid;
  const bool valid = my < samples;
  const int64_t myc = a.chain_off[inst] + (valid ? my : 0);
  float* H = Hs + tid;  // field of spin c at H[c * 128]
  for (int c = 0; c < 32; ++c)
    H[c * 128] = (valid && c < n) ? a.fields[myc * a.field_ld + c] : 0.0f;
  __syncthreads();
  if (!valid) return;
  const bool ising = a.problem_type == PYSA_GB_ISING;
  uint32_t word = a.spins[myc * a.words];
  double E = (double)a.energies[myc];
  int ones = __popc(word);
  double lw = 0.0;
  float beta_old = 0.0f;
  const double lr = a.ref == 1 ? log((1.0 - a.p) / a.p) : 0.0;
  const double logp = a.ref == 1 ? log(a.p) : 0.0;
  const double log1p_ = a.ref == 1 ? log(1.0 - a.p) : 0.0;
  for (int k = 0; k < a.num_temps; ++k) {
    const float beta = a.temps[k];
    if (a.order == 1) {
      lw += ais_dlw(beta, beta_old, (float)E, n, ones, logp, log1p_,
                    a.ref != 1);
    }
    const int32_t* perm =
        a.perm + ((int64_t)k * a.num_instances + inst) * a.max_n;
    uint32_t rnd[4];
    for (int t = 0; t < n; ++t) {
      if ((t & 3) == 0)
        draw4(a.seed, TAG_AIS, (uint32_t)inst, (uint32_t)k, (uint32_t)my,
              (uint32_t)(t >> 2), rnd);
      const uint32_t x = (t & 3) == 0 ? rnd[0] : (t & 3) == 1 ? rnd[1]
                         : (t & 3) == 2 ? rnd[2] : rnd[3];
      const int i = a.update == PYSA_GB_RANDOM ? perm[t] : t;
      const float hv = H[i * 128];
      const bool sbit = (word >> i) & 1u;
      const float dn = ising ? (sbit ? 2.0f * hv : -2.0f * hv)
                             : (sbit ? hv : -hv);
      const bool acc = ais_accept(beta, dn, sbit, lr, a.ref != 1, x);
      if (acc) {
        E -= (double)dn;
        ones += sbit ? -1 : 1;
        word ^= 1u << i;
      }
      const float d = acc ? (ising ? (sbit ? -2.0f : 2.0f)
                                   : (sbit ? -1.0f : 1.0f))
                          : 0.0f;
      const float* Jr = Js + i * 32;
#pragma unroll 8
      for (int c = 0; c < n; ++c) H[c * 128] = fmaf(d, Jr[c], H[c * 128]);
    }
    if (a.order == 0) {
      lw += ais_dlw(beta, beta_old, (float)E, n, ones, logp, log1p_,
                    a.ref != 1);
    }
    beta_old = beta;
  }
  a.log_w[myc] = lw;
  a.energies[myc] = (float)E;
  a.spins[myc * a.words] = word;
}

// Warp per sample keeps the code simple for the small n AIS is used on;
// GW samples per warp amortise the decision shuffles.
template <int NC, int GW>
static cudaError_t launch_ais_t(const AisArgs& a, int64_t max_samples,
                                cudaStream_t st) {
  const int64_t warps = (max_samples + GW - 1) / GW;
  const int64_t blocks = (warps * 32 + 127) / 128;
  dim3 grid((unsigned)(blocks > 0 ? blocks : 1), (unsigned)a.num_instances);
  k_ais<NC, GW><<<grid, 128, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_ais(const AisArgs& a, int64_t max_samples, cudaStream_t st) {
  if (a.max_n <= 32) {
    const int64_t blocks = (max_samples + 127) / 128;
    dim3 grid((unsigned)(blocks > 0 ? blocks : 1), (unsigned)a.num_instances);
    k_ais_small<<<grid, 128, 0, st>>>(a);
    return cudaGetLastError();
  }
  const int nc = (a.max_n + 31) / 32;
  if (nc <= 1) return launch_ais_t<1, 8>(a, max_samples, st);
  if (nc <= 2) return launch_ais_t<2, 8>(a, max_samples, st);
  if (nc <= 4) return launch_ais_t<4, 8>(a, max_samples, st);
  if (nc <= 8) return launch_ais_t<8, 4>(a, max_samples, st);
  if (nc <= 16) return launch_ais_t<16, 2>(a, max_samples, st);
  if (nc <= 32) return launch_ais_t<32, 1>(a, max_samples, st);
  return cudaErrorInvalidValue;
}

// Fisher-Yates of instance blockIdx.y for sweep blockIdx.x (draws of
// stream PERM, a = sweep), j = floor(x (i+1) / 2^32).
__global__ void k_perm_all(const int32_t* n_tab, int num_instances, int max_n,
                           uint64_t seed, int32_t* out) {
  extern __shared__ int32_t sh[];
  const int inst = blockIdx.y;
  const int n = n_tab[inst];
  const uint32_t sweep = blockIdx.x;
  int32_t* p = sh;
  uint32_t* x = reinterpret_cast<uint32_t*>(sh + max_n);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    p[i] = i;
    x[i] = draw1(seed, TAG_PERM, (uint32_t)inst, sweep, 0u, (uint32_t)i);
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = n - 1; i > 0; --i) {
      const int j = (int)(((uint64_t)x[i] * (uint64_t)(i + 1)) >> 32);
      const int32_t t = p[i];
      p[i] = p[j];
      p[j] = t;
    }
  __syncthreads();
  int32_t* o = out + ((int64_t)sweep * num_instances + inst) * max_n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) o[i] = p[i];
}

cudaError_t launch_perm_all(const int32_t* n_tab, int num_instances, int max_n,
                            int count, uint64_t seed, int32_t* out,
                            cudaStream_t st) {
  if (count <= 0 || num_instances <= 0) return cudaSuccess;
  dim3 grid((unsigned)count, (unsigned)num_instances);
  k_perm_all<<<grid, 256, sizeof(int32_t) * 2 * max_n, st>>>(
      n_tab, num_instances, max_n, seed, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- log Z
// Thread t of instance b walks Gray codes g(j), j in [t 2^B, (t+1) 2^B):
// fields and energy of the first state from scratch in f64, then one flip
// per step.  Per-thread (max, sum) of exp(-beta E) relative to the max.
__global__ void k_logz(const LogzArgs a) {
  const int inst = blockIdx.y;
  const int n = a.n[inst];
  const int ld = a.ld[inst];
  const float* J = a.J + a.j_off[inst];
  const float* h = a.h + a.h_off[inst];
  const int B = n < a.chunk_bits ? n : a.chunk_bits;
  const uint64_t threads = (uint64_t)1 << (n - B);
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double mx = -INFINITY, sum = 0.0;
  if (t < threads) {
    const bool ising = a.problem_type == PYSA_GB_ISING;
    const double lo = ising ? -1.0 : 0.0;
    double s[32], f[32];
    const uint64_t j0 = t << B;
    const uint64_t g0 = j0 ^ (j0 >> 1);
    for (int i = 0; i < n; ++i) s[i] = ((g0 >> i) & 1u) ? 1.0 : lo;
    double e = 0.0;
    for (int i = 0; i < n; ++i) {
      double acc = 0.0;
      for (int j = 0; j < n; ++j) acc += (double)J[(int64_t)i * ld + j] * s[j];
      f[i] = acc;
      e += s[i] * (0.5 * acc + (double)h[i]);
    }
    const double beta = a.beta;
    const uint64_t steps = (uint64_t)1 << B;
    for (uint64_t q = 0; q < steps; ++q) {
      const double w = -beta * e;
      if (w > mx) {
        sum = sum * exp(mx - w) + 1.0;
        mx = w;
      } else {
        sum += exp(w - mx);
      }
      if (q + 1 == steps) break;
      const int i = __ffsll((long long)(j0 + q + 1)) - 1;
      const double ns = ising ? -s[i] : 1.0 - s[i];
      const double d = ns - s[i];
      e += d * (f[i] + (double)h[i]);
      for (int j = 0; j < n; ++j) f[j] += (double)J[(int64_t)i * ld + j] * d;
      s[i] = ns;
    }
  }
  // block reduction of (max, sum)
  __shared__ double smx[256], ssum[256];
  smx[threadIdx.x] = mx;
  ssum[threadIdx.x] = sum;
  __syncthreads();
  for (int o = blockDim.x >> 1; o; o >>= 1) {
    if (threadIdx.x < o) {
      const double m1 = smx[threadIdx.x], m2 = smx[threadIdx.x + o];
      const double s1 = ssum[threadIdx.x], s2 = ssum[threadIdx.x + o];
      const double m = m1 > m2 ? m1 : m2;
      double v = 0.0;
      if (m1 != -INFINITY) v += s1 * exp(m1 - m);
      if (m2 != -INFINITY) v += s2 * exp(m2 - m);
      smx[threadIdx.x] = m;
      ssum[threadIdx.x] = v;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int64_t slot = (int64_t)inst * gridDim.x + blockIdx.x;
    a.part_max[slot] = smx[0];
    a.part_sum[slot] = ssum[0];
  }
}

cudaError_t launch_logz(const LogzArgs& a, int max_n, cudaStream_t st) {
  const int B = max_n < a.chunk_bits ? max_n : a.chunk_bits;
  const uint64_t threads = (uint64_t)1 << (max_n - B);
  const uint64_t blocks = (threads + 255) / 256;
  dim3 grid((unsigned)blocks, (unsigned)a.num_instances);
  k_logz<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace pysa_gb
