// kernels_aux.cu -- the kernels around the sweep: coupling packing, field and
// energy preparation, replica exchange + log-omega, visiting orders, f64
// energies and spin unpacking.
#include "aux.cuh"
#include "sweep_plain.cuh"

namespace pysa_gb {

// ------------------------------------------------------------ J packing
// packed[i][l * LS + m] = J[i][32 m + l] (0 outside the instance).
__global__ void k_pack_rows(const float* J, int ld, int n, int nc, int ls,
                            float* packed) {
  const int row_len = 32 * ls;
  const int64_t total = (int64_t)n * row_len;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / row_len), r = (int)(e % row_len);
    const int l = r / ls, m = r % ls;
    const int col = 32 * m + l;
    packed[e] = (m < nc && col < n) ? J[(int64_t)i * ld + col] : 0.0f;
  }
}

void launch_pack_rows(const float* J, int ld, int n, int nc, int ls,
                      float* packed, cudaStream_t st) {
  const int64_t total = (int64_t)n * 32 * ls;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  k_pack_rows<<<blocks, 256, 0, st>>>(J, ld, n, nc, ls, packed);
}

// -------------------------------------------------- fields and energies
// CTA per chain, warp per chunk of 256 columns (8 per lane).  F_i = sum_j
// J_ij s_j in f64, from f32 partial sums over 32 rows (the products J_ij s_j
// are exact in f32); H_i = f32(F_i + h_i); E = sum_i s_i (F_i / 2 + h_i)
// (pysa/ising.py:37, pysa/qubo.py:37), summed per lane, then over the warp,
// then over the chunks in order, so the result does not depend on timing.
constexpr int kFieldWarps = 8;

// Sparse instances: f_i = sum over row i's stored entries of J_ij s_j in f64
// (the products are exact; padding entries have value 0), from the fixed
// records (width > 0: entries csr_ent_off + width i ...) or the grouped
// rows (csr_rows, 9 offsets per row).
__device__ __forceinline__ double csr_row_dot(const pysa_gb_problems& p,
                                              int inst, int i,
                                              const uint32_t* sw,
                                              bool ising) {
  const int64_t eo = p.csr_ent_off[inst];
  int64_t beg, end;
  if (p.csr_width > 0) {
    beg = eo + (int64_t)p.csr_width * i;
    end = beg + p.csr_width;
  } else {
    const int32_t* r = p.csr_rows + 9 * (p.csr_row_off[inst] + i);
    beg = eo + r[0];
    end = eo + r[8];
  }
  double f = 0.0;
  for (int64_t e = beg; e < end; ++e) {
    const int j = p.csr_col[e] & 0x7fffffff;
    const float sj = ((sw[j >> 5] >> (j & 31)) & 1u) ? 1.0f
                                                     : (ising ? -1.0f : 0.0f);
    f += (double)(p.csr_val[e] * sj);
  }
  return f;
}

__device__ __forceinline__ bool is_sparse_inst(const pysa_gb_problems& p,
                                               int inst) {
  return p.csr_row_off && p.csr_row_off[inst] >= 0;
}

__global__ void __launch_bounds__(32 * kFieldWarps) k_fields(const PrepArgs a) {
  __shared__ double e_s[kFieldWarps];
  const int64_t c = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  // instance of chain c: binary search over chain_off
  int lo = 0, hi = a.p.num_instances - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (a.p.chain_off[mid] <= c) lo = mid; else hi = mid - 1;
  }
  const int inst = lo;
  const int n = a.p.n[inst], ld = a.p.ld[inst];
  const bool ising = a.p.problem_type == PYSA_GB_ISING;
  const float* J = a.p.J + a.p.j_off[inst];
  const float* h = a.p.h + a.p.h_off[inst];
  const uint32_t* sw = a.s.spins + c * a.p.words;
  double e = 0.0;
  if (is_sparse_inst(a.p, inst)) {  // uniform per CTA
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double f = csr_row_dot(a.p, inst, i, sw, ising);
      const uint32_t bit = (sw[i >> 5] >> (i & 31)) & 1u;
      const double si = bit ? 1.0 : (ising ? -1.0 : 0.0);
      e += si * (0.5 * f + (double)h[i]);
      a.fields[c * a.field_ld + i] = (float)(f + (double)h[i]);
    }
    e = warp_sum(e);
    if (lane == 0) e_s[warp] = e;
    __syncthreads();
    if (threadIdx.x == 0 && a.set_energies) {
      double t = 0.0;
      for (int w = 0; w < nwarps; ++w) t += e_s[w];
      a.s.energies[c] = (float)t;
    }
    return;
  }
  constexpr int TC = 8;  // columns per lane per chunk
  for (int base = 256 * warp; base < n; base += 256 * nwarps) {
    double F[TC];
    float part[TC];
#pragma unroll
    for (int k = 0; k < TC; ++k) {
      F[k] = 0.0;
      part[k] = 0.0f;
    }
    for (int j = 0; j < n; ++j) {
      const uint32_t bit = (sw[j >> 5] >> (j & 31)) & 1u;
      const float sj = bit ? 1.0f : (ising ? -1.0f : 0.0f);
      if (sj != 0.0f) {
        const float* row = J + (int64_t)j * ld;  // J symmetric: J[j][i]
#pragma unroll
        for (int k = 0; k < TC; ++k) {
          const int col = base + 32 * k + lane;
          if (col < n) part[k] += sj * row[col];
        }
      }
      if ((j & 31) == 31 || j == n - 1) {
#pragma unroll
        for (int k = 0; k < TC; ++k) {
          F[k] += (double)part[k];
          part[k] = 0.0f;
        }
      }
    }
    double ec = 0.0;
#pragma unroll
    for (int k = 0; k < TC; ++k) {
      const int col = base + 32 * k + lane;
      if (col < n) {
        const uint32_t bit = (sw[col >> 5] >> (col & 31)) & 1u;
        const double si = bit ? 1.0 : (ising ? -1.0 : 0.0);
        ec += si * (0.5 * F[k] + (double)h[col]);
        a.fields[c * a.field_ld + col] = (float)(F[k] + (double)h[col]);
      }
    }
    e += warp_sum(ec);
  }
  if (lane == 0) e_s[warp] = e;
  __syncthreads();
  if (threadIdx.x == 0 && a.set_energies) {
    double t = 0.0;
    for (int w = 0; w < nwarps; ++w) t += e_s[w];
    a.s.energies[c] = (float)t;
  }
}

// CTA per read, thread per replica: the slot betas and the initial best.
__global__ void k_read_init(const PrepArgs a) {
  const int64_t r = blockIdx.x;
  const int inst = a.p.read_inst[r];
  const int R = a.p.replicas[inst];
  const int64_t base = a.p.chain_off[inst] + (r - a.p.read_off[inst]) * R;
  const float* betas = a.p.ladder + a.p.ladder_off[inst];
  for (int k = threadIdx.x; k < R; k += blockDim.x) {
    a.s.chain_beta[base + a.s.beta_idx[base + k]] = betas[k];
    if (a.init_best) {
      const int64_t c = base + k;
      a.s.best_energy[c] = a.best_global ? __int_as_float(0x7f800000)
                                         : a.s.energies[c];
      a.s.best_sweep[c] = 0;
      for (int w = 0; w < a.p.words; ++w)
        a.s.best_spins[c * a.p.words + w] = a.s.spins[c * a.p.words + w];
    }
  }
}

void launch_prepare(const PrepArgs& a, cudaStream_t st) {
  if (a.p.num_chains > 0) {
    int warps = (a.p.max_n + 255) / 256;
    warps = warps < 1 ? 1 : warps > kFieldWarps ? kFieldWarps : warps;
    k_fields<<<(unsigned)a.p.num_chains, warps * 32, 0, st>>>(a);
  }
  if (a.p.num_reads > 0)
    k_read_init<<<(unsigned)a.p.num_reads, 128, 0, st>>>(a);
}

// ------------------------------------------------------ replica exchange
// Warp per read.  pysa/utils.py:44-58: pairs (R-1,R-2), (R-2,R-3), ... in
// order; swap beta_idx when de >= 0 or u < exp(de), de in f32.  Then the
// per-replica betas of the next sweep and, if requested, get_log_omega
// (pysa/ais.py:79-112) in f64.  The last block to finish advances the sweep
// counter.
constexpr int kXWarps = 4;


__global__ void k_exchange(const XArgs a) {
  __shared__ float E_s[kXWarps][kMaxReplicas];
  __shared__ int32_t B_s[kXWarps][kMaxReplicas];
  __shared__ uint32_t X_s[kXWarps][kMaxReplicas];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * kXWarps + warp;
  const uint32_t sweep = (uint32_t)(*a.s.sweep_counter);
  const bool xch = a.use_pt && exchange_after(a.exchange_every, sweep);
  if (r < a.p.num_reads) {
    const int inst = a.p.read_inst[r];
    const int R = a.p.replicas[inst];
    const int64_t lread = r - a.p.read_off[inst];
    const int64_t base = a.p.chain_off[inst] + lread * R;
    const float* betas = a.p.ladder + a.p.ladder_off[inst];
    float* E = E_s[warp];
    int32_t* B = B_s[warp];
    uint32_t* X = X_s[warp];
    for (int k = lane; k < R; k += 32) {
      E[k] = a.s.energies[base + k];
      B[k] = a.s.beta_idx[base + k];
      if (xch && k < R - 1)
        X[k] = draw1(a.seed, TAG_PT, (uint32_t)inst, sweep, (uint32_t)lread,
                     (uint32_t)k);
    }
    __syncwarp();
    if (xch && R > 1 && lane == 0) {
      for (int k = 0; k < R - 1; ++k) {
        const int k1 = R - k - 1, k2 = R - k - 2;
        const int b1 = B[k1], b2 = B[k2];
        const float de = __fmul_rn(__fsub_rn(E[b1], E[b2]),
                                   __fsub_rn(betas[k1], betas[k2]));
        if (pt_accept(de, X[k])) {
          B[k1] = b2;
          B[k2] = b1;
        }
      }
    }
    __syncwarp();
    for (int k = lane; k < R; k += 32) {
      a.s.beta_idx[base + k] = B[k];
      a.s.chain_beta[base + B[k]] = betas[k];
    }
    if (a.log_omega_stride > 0 && lane == 0) {
      const int32_t* sorted = a.p.ladder_sorted + a.p.ladder_off[inst];
      double lw = 0.0;
      float beta_old = 0.0f;
      for (int q = 1; q < R; ++q) {
        const float b = betas[sorted[q]];
        const float e = E[B[sorted[q]]];
        const float t1 = __fmul_rn(-b, e), t2 = __fmul_rn(-beta_old, e);
        lw += (double)__fsub_rn(t1, t2);
        beta_old = b;
      }
      a.s.log_omega[r * a.log_omega_stride + sweep] = lw;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const uint32_t t = atomicAdd(a.s.ticket, 1u);
    if (t == gridDim.x - 1) {
      *a.s.ticket = 0u;
      __threadfence();
      *a.s.sweep_counter += 1;
    }
  }
}

void launch_exchange(const XArgs& a, cudaStream_t st) {
  const int64_t blocks = (a.p.num_reads + kXWarps - 1) / kXWarps;
  k_exchange<<<(unsigned)(blocks > 0 ? blocks : 1), kXWarps * 32, 0, st>>>(a);
}

// ---------------------------------------------------- visiting orders
// Fisher-Yates for (instance, sweep): j = floor(x (i+1) / 2^32); draws made
// in parallel, swaps by one thread.  Block per instance.
__global__ void k_perm(const PermArgs a) {
  extern __shared__ int32_t sh[];
  const int inst = blockIdx.x;
  const int n = a.p.n[inst];
  // grid row y: the sweep y after the current one (orders made ahead)
  const uint32_t sweep = (uint32_t)(*a.sweep_counter) + blockIdx.y;
  int32_t* p = sh;
  uint32_t* x = reinterpret_cast<uint32_t*>(sh + a.p.max_n);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    p[i] = i;
    x[i] = draw1(a.seed, TAG_PERM, (uint32_t)inst, sweep, 0u, (uint32_t)i);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = n - 1; i > 0; --i) {
      const int j = (int)(((uint64_t)x[i] * (uint64_t)(i + 1)) >> 32);
      const int32_t t = p[i];
      p[i] = p[j];
      p[j] = t;
    }
  }
  __syncthreads();
  int32_t* out = a.perm + ((int64_t)(sweep % (uint32_t)a.perm_slots) *
                               a.p.num_instances + inst) * (int64_t)a.p.max_n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = p[i];
}

// The same orders for instances too wide for k_perm's shared memory (up to
// 65536 spins): the draws are staged in the output row, the positions held
// as 16-bit values in shared memory.
__global__ void k_perm_wide(const PermArgs a) {
  extern __shared__ uint16_t pw[];
  const int inst = blockIdx.x;
  const int n = a.p.n[inst];
  const uint32_t sweep = (uint32_t)(*a.sweep_counter) + blockIdx.y;
  int32_t* out = a.perm + ((int64_t)(sweep % (uint32_t)a.perm_slots) *
                               a.p.num_instances + inst) * (int64_t)a.p.max_n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    pw[i] = (uint16_t)i;
    out[i] = (int32_t)draw1(a.seed, TAG_PERM, (uint32_t)inst, sweep, 0u,
                            (uint32_t)i);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = n - 1; i > 0; --i) {
      const uint32_t xi = (uint32_t)__ldcg(out + i);
      const int j = (int)(((uint64_t)xi * (uint64_t)(i + 1)) >> 32);
      const uint16_t t = pw[i];
      pw[i] = pw[j];
      pw[j] = t;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = (int32_t)pw[i];
}

void launch_perm(const PermArgs& a, cudaStream_t st, int count) {
  const size_t sm = sizeof(int32_t) * 2 * (size_t)a.p.max_n;
  dim3 grid((unsigned)a.p.num_instances, (unsigned)(count > 0 ? count : 1));
  if (sm <= 48 * 1024) {
    k_perm<<<grid, 256, sm, st>>>(a);
    return;
  }
  const size_t smw = sizeof(uint16_t) * (size_t)a.p.max_n;  // <= 128 KB
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    cudaFuncSetAttribute(k_perm_wide,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(uint16_t) * PYSA_GB_MAX_N));
    attr[dev] = true;
  }
  k_perm_wide<<<grid, 256, smw, st>>>(a);
}

// ----------------------------------------------------------- f64 energy
// CTA per state, warp per row i (rows warp, warp + 8, ...), lanes over the
// columns: f_i = sum_j J_ij s_j, E = sum_i s_i (f_i / 2 + h_i) in f64,
// reduced in a fixed order (lanes, then rows of a warp, then warps).
template <typename T>
__device__ __forceinline__ void energy64_body(
    int ptype, int n, int ld, const T* J, const T* h, const uint32_t* spins,
    int words, double* out) {
  __shared__ double e_s[8];
  const int64_t c = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t* sw = spins + c * words;
  const bool ising = ptype == PYSA_GB_ISING;
  double e = 0.0;
  for (int i = warp; i < n; i += 8) {
    const double si =
        ((sw[i >> 5] >> (i & 31)) & 1u) ? 1.0 : (ising ? -1.0 : 0.0);
    if (si == 0.0) continue;  // warp-uniform
    const T* row = J + (int64_t)i * ld;
    double f = 0.0;
    for (int j = lane; j < n; j += 32) {
      const double sj =
          ((sw[j >> 5] >> (j & 31)) & 1u) ? 1.0 : (ising ? -1.0 : 0.0);
      f += (double)row[j] * sj;
    }
    f = warp_sum(f);
    e += si * (0.5 * f + (double)h[i]);
  }
  if (lane == 0) e_s[warp] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += e_s[w];
    out[c] = t;
  }
}

__global__ void __launch_bounds__(256) k_energy64(
    int ptype, int n, int ld, const double* J, const double* h,
    const uint32_t* spins, int words, double* out) {
  energy64_body<double>(ptype, n, ld, J, h, spins, words, out);
}

// Same with instance inst's f32 couplings and fields of the problem tables.
// Sparse instances from their stored rows (thread per row, fixed
// reduction order).
__global__ void __launch_bounds__(256) k_energy64_tables(
    const pysa_gb_problems p, int inst, const uint32_t* spins, int words,
    double* out) {
  if (!is_sparse_inst(p, inst)) {
    energy64_body<float>(p.problem_type, p.n[inst], p.ld[inst],
                         p.J + p.j_off[inst], p.h + p.h_off[inst], spins,
                         words, out);
    return;
  }
  __shared__ double e_s[8];
  const int64_t c = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t* sw = spins + c * words;
  const bool ising = p.problem_type == PYSA_GB_ISING;
  const int n = p.n[inst];
  const float* h = p.h + p.h_off[inst];
  double e = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double si =
        ((sw[i >> 5] >> (i & 31)) & 1u) ? 1.0 : (ising ? -1.0 : 0.0);
    if (si != 0.0) e += si * (0.5 * csr_row_dot(p, inst, i, sw, ising) +
                              (double)h[i]);
  }
  e = warp_sum(e);
  if (lane == 0) e_s[warp] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += e_s[w];
    out[c] = t;
  }
}

void launch_energy64(int ptype, int n, int ld, const double* J,
                     const double* h, const uint32_t* spins, int words,
                     int64_t count, double* out, cudaStream_t st) {
  if (count > 0)
    k_energy64<<<(unsigned)count, 256, 0, st>>>(ptype, n, ld, J, h, spins,
                                                words, out);
}

void launch_energy64_tables(const pysa_gb_problems& p, int inst,
                            const uint32_t* spins, int words, int64_t count,
                            double* out, cudaStream_t st) {
  if (count > 0)
    k_energy64_tables<<<(unsigned)count, 256, 0, st>>>(p, inst, spins, words,
                                                       out);
}

// ---------------------------------------------------------------- unpack
__global__ void k_unpack(int ptype, int n, const uint32_t* spins, int words,
                         int64_t count, float* out, int out_ld) {
  const int64_t total = count * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / n;
    const int j = (int)(e % n);
    const uint32_t bit = (spins[c * words + (j >> 5)] >> (j & 31)) & 1u;
    out[c * out_ld + j] = bit ? 1.0f : (ptype == PYSA_GB_ISING ? -1.0f : 0.0f);
  }
}

void launch_unpack(int ptype, int n, const uint32_t* spins, int words,
                   int64_t count, float* out, int out_ld, cudaStream_t st) {
  const int64_t total = count * n;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 65535) blocks = 65535;
  if (blocks > 0)
    k_unpack<<<(unsigned)blocks, 256, 0, st>>>(ptype, n, spins, words, count,
                                               out, out_ld);
}

// Float states (+-1 or 0/1) -> bit-packed words: a warp per (state, word),
// one ballot per word.  The bit is x > 0 (Ising) or x != 0 (QUBO), the rule
// of the host-side packing.
__global__ void k_pack(int ptype, int n, const float* x, int x_ld,
                       int64_t count, uint32_t* spins, int words) {
  const int lane = threadIdx.x & 31;
  const int64_t total = count * words;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t e = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
       e < total; e += nw) {
    const int64_t c = e / words;
    const int w = (int)(e % words);
    const int j = 32 * w + lane;
    bool b = false;
    if (j < n) {
      const float v = x[c * x_ld + j];
      b = ptype == PYSA_GB_ISING ? v > 0.0f : v != 0.0f;
    }
    const uint32_t bits = __ballot_sync(0xffffffffu, b);
    if (lane == 0) spins[c * words + w] = bits;
  }
}

void launch_pack(int ptype, int n, const float* x, int x_ld, int64_t count,
                 uint32_t* spins, int words, cudaStream_t st) {
  const int64_t warps = count * words;
  int64_t blocks = (warps + 7) / 8;
  if (blocks > 65535) blocks = 65535;
  if (blocks > 0)
    k_pack<<<(unsigned)blocks, 256, 0, st>>>(ptype, n, x, x_ld, count, spins,
                                             words);
}

// A dense symmetric problem matrix P (n x n, row stride p_ld) of instance
// inst split as the reference's Solver does (pysa/sa.py:66-69): couplings =
// P with a zero diagonal, stored transposed (row j = column j of P), and
// local fields = diag(P).
__global__ void k_load_problem(const pysa_gb_problems p, int inst,
                               const float* P, int p_ld) {
  const int n = p.n[inst];
  const int ld = p.ld[inst];
  // the tables' J and h are const for the sweeps; this kernel refills them
  float* Jt = const_cast<float*>(p.J) + p.j_off[inst];
  float* h = const_cast<float*>(p.h) + p.h_off[inst];
  const int64_t total = (int64_t)n * ld;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / ld), i = (int)(e % ld);
    float v = 0.0f;
    if (i < n && i != j) v = P[(int64_t)i * p_ld + j];
    Jt[e] = v;
    if (i == j) h[j] = P[(int64_t)j * p_ld + j];
  }
}

void launch_load_problem(const pysa_gb_problems& p, int inst, int n, int ld,
                         const float* P, int p_ld, cudaStream_t st) {
  const int64_t total = (int64_t)n * ld;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 65535) blocks = 65535;
  if (blocks > 0)
    k_load_problem<<<(unsigned)blocks, 256, 0, st>>>(p, inst, P, p_ld);
}

}  // namespace pysa_gb
