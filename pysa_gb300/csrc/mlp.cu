// mlp.cu -- learned flip proposal: per-instance MLP n -> hidden -> n
// (Bernoulli flip logits), its training (forward, backward, Adam) and the
// Metropolis-Hastings proposal step, all on the GPU.
//
// No counterpart in the reference.  The GEMMs run on k_gemm_tc (tcgen05,
// BF16 operands, FP32 accumulation); everything else is elementwise or
// row-reduction kernels written here.  FP32 master weights, BF16 packed
// copies for the tensor cores.
//
// Proposal for a chain in state s (values +-1 or 0/1):
//   p = sigmoid(MLP(s));  flip mask f_j ~ Bernoulli(p_j);  s' = s flipped on f
//   log q(s'|s) = sum_j [f_j log p_j + (1 - f_j) log(1 - p_j)]
//   log q(s|s') = same mask under p' = sigmoid(MLP(s'))
//   dE = E(s') - E(s) = 1/2 delta.(H + H'),  H' = H + J delta  (exact for
//   integer couplings), delta = s' - s
//   accept iff log u < -beta dE + log q(s|s') - log q(s'|s)
// which satisfies detailed balance for exp(-beta E).
#include "aux.cuh"
#include "gemm_api.h"
#include "plain_variants.h"

namespace pysa_gb {

// ---------------------------------------------------------- elementwise
// dz2 = w_r (sigmoid(z2) - f) / sum(w); loss += w_r BCE / sum(w)
__global__ void k_bce_grad(const float* z2, const float* f, const float* w,
                           int B, int n, float* dz2, float* loss) {
  const int i = blockIdx.y;
  const int64_t off = (int64_t)i * B * n;
  float wsum = 0.0f;
  for (int r = 0; r < B; ++r) wsum += w[(int64_t)i * B + r];
  const float inv = wsum > 0.0f ? 1.0f / wsum : 0.0f;
  float acc = 0.0f;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       e < (int64_t)B * n; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / n);
    const float wr = w[(int64_t)i * B + r] * inv;
    const float z = z2[off + e], t = f[off + e];
    const float p = 1.0f / (1.0f + __expf(-z));
    dz2[off + e] = wr * (p - t);
    // BCE with logits: max(z,0) - z t + log(1 + exp(-|z|))
    acc += wr * (fmaxf(z, 0.0f) - z * t + log1pf(__expf(-fabsf(z))));
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss + i, acc);
}

// dz1 = da1 * (a1 > 0), in place
__global__ void k_relu_mask(float* da1, const float* a1, int64_t total) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x)
    if (a1[e] <= 0.0f) da1[e] = 0.0f;
}

// column sums of [B][cols] per instance -> out[i][cols]
__global__ void k_colsum(const float* x, int B, int cols, float* out) {
  const int i = blockIdx.y;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const float* xi = x + (int64_t)i * B * cols;
  float s = 0.0f;
  for (int r = 0; r < B; ++r) s += xi[(int64_t)r * cols + c];
  out[(int64_t)i * cols + c] = s;
}

// Adam (Kingma & Ba) on FP32 masters: m = b1 m + (1-b1) g, v = b2 v +
// (1-b2) g^2, w -= lr * mhat / (sqrt(vhat) + eps).
__global__ void k_adam(float* w, float* m, float* v, const float* g,
                       int64_t total, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const float gr = g[e];
    const float mm = b1 * m[e] + (1.0f - b1) * gr;
    const float vv = b2 * v[e] + (1.0f - b2) * gr * gr;
    m[e] = mm;
    v[e] = vv;
    w[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
  }
}

// ------------------------------------------------------------- proposals
// rows[i][r] = chain of read r of instance i holding the largest beta (first
// replica on ties), -1 beyond the instance's reads or for disabled instances.
__global__ void k_cold_rows(const pysa_gb_problems p, const float* chain_beta,
                            const int32_t* enabled, int B, int32_t* rows) {
  const int i = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= B) return;
  const int R = p.replicas[i], Rd = p.reads[i];
  int32_t c = -1;
  if (r < Rd && (!enabled || enabled[i])) {
    const int64_t base = p.chain_off[i] + (int64_t)r * R;
    float bmax = chain_beta[base];
    int64_t arg = base;
    for (int k = 1; k < R; ++k) {
      const float b = chain_beta[base + k];
      if (b > bmax) {
        bmax = b;
        arg = base + k;
      }
    }
    c = (int32_t)arg;
  }
  rows[(int64_t)i * B + r] = c;
}

// x[i][r][j] = spin j of chain rows[i][r] as +-1 / 0 1 (0 for padding).
__global__ void k_gather_rows(const pysa_gb_problems p, const uint32_t* spins,
                              const int32_t* rows, int B, int nn, float* x) {
  const int i = blockIdx.y;
  const int n_i = p.n[i];
  const bool ising = p.problem_type == PYSA_GB_ISING;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       e < (int64_t)B * nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / nn), j = (int)(e % nn);
    const int32_t c = rows[(int64_t)i * B + r];
    float v = 0.0f;
    if (c >= 0 && j < n_i) {
      const uint32_t bit = (spins[(int64_t)c * p.words + (j >> 5)] >> (j & 31)) & 1u;
      v = bit ? 1.0f : (ising ? -1.0f : 0.0f);
    }
    x[((int64_t)i * B + r) * nn + j] = v;
  }
}

// log sigmoid(z) and log(1 - sigmoid(z)) = log sigmoid(-z), stable form
// -softplus(-z) = -(max(-z, 0) + log1p(exp(-|z|))).
__device__ __forceinline__ float log_sigmoid(float z) {
  return -(fmaxf(-z, 0.0f) + log1pf(expf(-fabsf(z))));
}

// Proposal-size control: the shift c with sum_{j<n} sigmoid(z_j + c) = k,
// by 40 bisection steps on [-60, 60] (c saturates at the ends when k is out
// of reach).  Warp-collective and a deterministic function of z, so the
// forward and the reverse pass use the same rule.  k <= 0: no shift.
__device__ float flip_shift(const float* z, int n, float k, int lane) {
  if (k <= 0.0f) return 0.0f;
  float lo = -60.0f, hi = 60.0f;
  for (int it = 0; it < 40; ++it) {
    const float c = 0.5f * (lo + hi);
    float sum = 0.0f;
    for (int j = lane; j < n; j += 32) sum += 1.0f / (1.0f + expf(-(z[j] + c)));
    sum = warp_sum(sum);
    if (sum > k)
      hi = c;
    else
      lo = c;
  }
  return 0.5f * (lo + hi);
}

// Warp per row: sample the flip mask from sigmoid(z + c) (c from
// flip_shift), log q(s'|s), and the proposed state x' (written over x) with
// delta = x' - x.  Flip j iff u < sigmoid(z_j + c), u = f32 of the uniform
// of stream (PROPOSAL, inst, round, chain, j).
__global__ void k_sample_flips(const pysa_gb_problems p, const int32_t* rows,
                               int B, int nn, const float* z, float* x,
                               float* flip, float* delta, float* logq,
                               uint64_t seed, uint32_t round, float k_flips) {
  const int i = blockIdx.y;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= B) return;
  const int32_t c = rows[(int64_t)i * B + r];
  const int n_i = p.n[i];
  const bool ising = p.problem_type == PYSA_GB_ISING;
  const int64_t o = ((int64_t)i * B + r) * nn;
  const float shift = c >= 0 ? flip_shift(z + o, n_i, k_flips, lane) : 0.0f;
  float lq = 0.0f;
  for (int j = lane; j < nn; j += 32) {
    float f = 0.0f, d = 0.0f;
    if (c >= 0 && j < n_i) {
      const float zz = z[o + j] + shift;
      const float u = (float)uniform64(draw1(seed, TAG_PROPOSAL, (uint32_t)i,
                                             round, (uint32_t)c, (uint32_t)j));
      const float pj = 1.0f / (1.0f + expf(-zz));
      f = u < pj ? 1.0f : 0.0f;
      lq += f > 0.0f ? log_sigmoid(zz) : log_sigmoid(-zz);
      if (f > 0.0f) {
        const float xv = x[o + j];
        const float xn = ising ? -xv : 1.0f - xv;
        d = xn - xv;
        x[o + j] = xn;
      }
    }
    flip[o + j] = f;
    delta[o + j] = d;
  }
  lq = warp_sum(lq);
  if (lane == 0) logq[(int64_t)i * B + r] = lq;
}

// log q(s|s') of the same mask under the logits at s'.
__global__ void k_logq_reverse(const int32_t* rows, int B, int nn,
                               const int32_t* n_inst, const float* z,
                               const float* flip, float* logq,
                               float k_flips) {
  const int i = blockIdx.y;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= B) return;
  const int n_i = n_inst[i];
  const int64_t o = ((int64_t)i * B + r) * nn;
  float lq = 0.0f;
  if (rows[(int64_t)i * B + r] >= 0) {
    const float shift = flip_shift(z + o, n_i, k_flips, lane);
    for (int j = lane; j < n_i; j += 32) {
      const float zz = z[o + j] + shift;
      lq += flip[o + j] > 0.0f ? log_sigmoid(zz) : log_sigmoid(-zz);
    }
  }
  lq = warp_sum(lq);
  if (lane == 0) logq[(int64_t)i * B + r] = lq;
}

// Warp per row: dE = delta.(H + J delta / 2) from the fields H and jd =
// J delta, Metropolis-Hastings decision, and on acceptance the new spins,
// fields, energy and (on a strict improvement) best state.
__global__ void k_mh_accept(const pysa_gb_problems p, pysa_gb_state s,
                            float* fields, int field_ld, const int32_t* rows,
                            int B, int nn, const float* x_new,
                            const float* delta, const float* jd,
                            const float* logq_fwd, const float* logq_rev,
                            uint64_t seed, uint32_t round, int32_t* accepted,
                            float* de_out) {
  const int i = blockIdx.y;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= B) return;
  const int64_t ir = (int64_t)i * B + r;
  const int32_t c = rows[ir];
  if (c < 0) {
    if (lane == 0) de_out[ir] = 0.0f;
    return;
  }
  const int n_i = p.n[i];
  const int64_t o = ir * nn;
  float* H = fields + (int64_t)c * field_ld;
  float de = 0.0f, nflip = 0.0f;
  for (int j = lane; j < n_i; j += 32) {
    const float d = delta[o + j];
    de += d * (H[j] + 0.5f * jd[o + j]);
    nflip += d != 0.0f ? 1.0f : 0.0f;
  }
  de = warp_sum(de);
  nflip = warp_sum(nflip);
  const float beta = s.chain_beta[c];
  const double loga = -(double)beta * (double)de + (double)logq_rev[ir] -
                      (double)logq_fwd[ir];
  const uint32_t xu = draw1(seed, TAG_PROPOSAL, (uint32_t)i, round,
                            (uint32_t)c, 0xFFFFFFFFu);
  const bool acc = nflip > 0.0f && (loga >= 0.0 || log(uniform64(xu)) < loga);
  if (lane == 0) de_out[ir] = acc ? de : 0.0f;
  if (!acc) return;
  const float e_new = s.energies[c] + de;
  const bool improved = e_new < s.best_energy[c];
  __syncwarp();
  for (int j = lane; j < n_i; j += 32) H[j] += jd[o + j];
  for (int w = lane; w < p.words; w += 32) {
    uint32_t word = 0;
    for (int b = 0; b < 32; ++b) {
      const int j = 32 * w + b;
      if (j < n_i && x_new[o + j] > 0.0f) word |= 1u << b;
    }
    s.spins[(int64_t)c * p.words + w] = word;
    if (improved) s.best_spins[(int64_t)c * p.words + w] = word;
  }
  if (lane == 0) {
    s.energies[c] = e_new;
    if (s.stream_key) s.stream_key[c] += 1u;  // fresh sweep stream
    if (improved) {
      s.best_energy[c] = e_new;
      const int64_t sw = *s.sweep_counter;
      s.best_sweep[c] = (int32_t)(sw > 0 ? sw - 1 : 0);
    }
    atomicAdd(accepted + i, 1);
  }
}

// B operand of J delta: out(row j, k) = J_field[j][k] = Jt[k][j] (the
// couplings are stored transposed, row k = change of every field when spin k
// flips), tiled K-major like k_pack_kmajor, zero-padded to nn x nn; term 0 =
// bf16(J), term 1 = bf16(J - bf16(J)).
__global__ void k_pack_proposal_j(const float* Jt, int n, int ld, int nn,
                                  int term, uint16_t* dst) {
  const int64_t total = (int64_t)nn * nn;
  const int kt_n = nn / 64;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = e / (256 * 64);
    const int within = (int)(e % (256 * 64));
    const int rt = (int)(t / kt_n), kt = (int)(t % kt_n);
    const int cm = within / 64, inside = within % 64;
    const int j = rt * 256 + (cm / 8) * 8 + inside / 8;
    const int k = kt * 64 + (cm % 8) * 8 + inside % 8;
    float v = (j < n && k < n) ? Jt[(int64_t)k * ld + j] : 0.0f;
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    if (term == 1) v -= __bfloat162float(hi);
    const __nv_bfloat16 h = term == 1 ? __float2bfloat16_rn(v) : hi;
    dst[e] = *reinterpret_cast<const uint16_t*>(&h);
  }
}

// Training pair from two snapshots of bit-packed cold states:
// x = state a (+-1 / 0 1), target f = (a != b).
__global__ void k_pairs(const uint32_t* a, const uint32_t* b, int words,
                        const int32_t* n_inst, int B, int nn, int ptype,
                        float* x, float* f) {
  const int i = blockIdx.y;
  const int n_i = n_inst[i];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       e < (int64_t)B * nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / nn), j = (int)(e % nn);
    const int64_t wi = ((int64_t)i * B + r) * words + (j >> 5);
    float xv = 0.0f, fv = 0.0f;
    if (j < n_i) {
      const uint32_t ba = (a[wi] >> (j & 31)) & 1u;
      const uint32_t bb = (b[wi] >> (j & 31)) & 1u;
      xv = ba ? 1.0f : (ptype == PYSA_GB_ISING ? -1.0f : 0.0f);
      fv = ba != bb ? 1.0f : 0.0f;
    }
    x[((int64_t)i * B + r) * nn + j] = xv;
    f[((int64_t)i * B + r) * nn + j] = fv;
  }
}

// Snapshot: words of the chains in rows -> out[i][r][words] (0 for -1).
__global__ void k_snapshot(const uint32_t* spins, int words, const int32_t* rows,
                           int B, int I, uint32_t* out) {
  const int64_t total = (int64_t)I * B * words;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ir = e / words;
    const int w = (int)(e % words);
    const int32_t c = rows[ir];
    out[e] = c >= 0 ? spins[(int64_t)c * words + w] : 0u;
  }
}

}  // namespace pysa_gb

// ====================================================================== ABI
using namespace pysa_gb;

namespace {
inline int grid_for(int64_t total) {
  int64_t b = (total + 255) / 256;
  if (b > 4096) b = 4096;
  if (b < 1) b = 1;
  return (int)b;
}

inline bool mlp_ok(const pysa_gb_mlp* m) {
  return m && m->num_instances > 0 && m->n > 0 && m->hidden > 0 &&
         m->batch > 0 && m->n % 256 == 0 && m->hidden % 256 == 0 &&
         m->batch % 128 == 0;
}

cudaError_t gemm(const pysa_gb_mlp* m, const uint16_t* A, int64_t sA,
                 const uint16_t* B, int64_t sB, float* C, int64_t sC, int ldc,
                 const float* bias, int64_t sBias, int M, int N, int K,
                 int relu, cudaStream_t st) {
  GemmArgs g;
  g.A = A;
  g.B = B;
  g.C = C;
  g.bias = bias;
  g.status = m->status;
  g.strideA = sA;
  g.strideB = sB;
  g.strideC = sC;
  g.strideBias = sBias;
  g.M = M;
  g.N = N;
  g.K = K;
  g.ldc = ldc;
  g.accumulate = 0;
  g.relu = relu;
  return launch_gemm_tc(g, m->num_instances, st);
}

cudaError_t pack(const pysa_gb_mlp* m, const float* src, int ld,
                 int64_t src_stride, int rows, int K, int transpose,
                 int tile_rows, uint16_t* dst, cudaStream_t st) {
  return launch_pack_kmajor(src, ld, src_stride, rows, K, transpose,
                            tile_rows, dst, (int64_t)rows * K,
                            m->num_instances, st);
}

cudaError_t mlp_forward(const pysa_gb_mlp* m, cudaStream_t st) {
  const int B = m->batch, n = m->n, H = m->hidden;
  cudaError_t e;
  // a1 = relu(x W1^T + b1)
  if ((e = pack(m, m->x, n, (int64_t)B * n, B, n, 0, 128, m->pa, st))) return e;
  if ((e = gemm(m, m->pa, (int64_t)B * n, m->w1_p, (int64_t)H * n, m->a1,
                (int64_t)B * H, H, m->b1, H, B, H, n, 1, st)))
    return e;
  // z2 = a1 W2^T + b2
  if ((e = pack(m, m->a1, H, (int64_t)B * H, B, H, 0, 128, m->pa, st))) return e;
  return gemm(m, m->pa, (int64_t)B * H, m->w2_p, (int64_t)n * H, m->z2,
              (int64_t)B * n, n, m->b2, n, B, n, H, 0, st);
}

cudaError_t mlp_repack(const pysa_gb_mlp* m, cudaStream_t st) {
  const int n = m->n, H = m->hidden;
  cudaError_t e;
  if ((e = pack(m, m->w1, n, (int64_t)H * n, H, n, 0, 256, m->w1_p, st)))
    return e;
  if ((e = pack(m, m->w2, H, (int64_t)n * H, n, H, 0, 256, m->w2_p, st)))
    return e;
  // W2^T as the B operand of dA1 = dZ2 W2: rows H, K n
  return pack(m, m->w2, H, (int64_t)n * H, H, n, 1, 256, m->w2t_p, st);
}
}  // namespace

static int mlp_fail(const char* what) {
  return pysa_gb_internal_fail(PYSA_GB_ERR_ARG, what);
}

static int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? PYSA_GB_OK
                          : pysa_gb_internal_fail(PYSA_GB_ERR_CUDA, what);
}

extern "C" {

int pysa_gb_mlp_sync_weights(const pysa_gb_mlp* m, void* stream) {
  if (!mlp_ok(m)) return mlp_fail("mlp: bad descriptor");
  return cuda_check(mlp_repack(m, (cudaStream_t)stream), "mlp repack");
}

int pysa_gb_mlp_forward(const pysa_gb_mlp* m, void* stream) {
  if (!mlp_ok(m)) return mlp_fail("mlp: bad descriptor");
  return cuda_check(mlp_forward(m, (cudaStream_t)stream), "mlp forward");
}

int pysa_gb_mlp_backward(const pysa_gb_mlp* m, const float* target,
                         const float* row_weight, void* stream) {
  if (!mlp_ok(m) || !target || !row_weight)
    return mlp_fail("mlp backward: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int B = m->batch, n = m->n, H = m->hidden, I = m->num_instances;
  cudaError_t e = cudaMemsetAsync(m->loss, 0, sizeof(float) * I, st);
  if (e) return cuda_check(e, "mlp loss reset");
  k_bce_grad<<<dim3(64, I), 256, 0, st>>>(m->z2, target, row_weight, B, n,
                                          m->dz2, m->loss);
  // dW2 = dZ2^T A1: M = n, N = H, K = B
  if ((e = pack(m, m->dz2, n, (int64_t)B * n, n, B, 1, 128, m->pa, st)) ||
      (e = pack(m, m->a1, H, (int64_t)B * H, H, B, 1, 256, m->pb, st)) ||
      (e = gemm(m, m->pa, (int64_t)n * B, m->pb, (int64_t)H * B, m->dw2,
                (int64_t)n * H, H, nullptr, 0, n, H, B, 0, st)))
    return cuda_check(e, "mlp dW2");
  // dA1 = dZ2 W2: M = B, N = H, K = n
  if ((e = pack(m, m->dz2, n, (int64_t)B * n, B, n, 0, 128, m->pa, st)) ||
      (e = gemm(m, m->pa, (int64_t)B * n, m->w2t_p, (int64_t)H * n, m->da1,
                (int64_t)B * H, H, nullptr, 0, B, H, n, 0, st)))
    return cuda_check(e, "mlp dA1");
  k_relu_mask<<<grid_for((int64_t)I * B * H), 256, 0, st>>>(
      m->da1, m->a1, (int64_t)I * B * H);
  // dW1 = dZ1^T X: M = H, N = n, K = B
  if ((e = pack(m, m->da1, H, (int64_t)B * H, H, B, 1, 128, m->pa, st)) ||
      (e = pack(m, m->x, n, (int64_t)B * n, n, B, 1, 256, m->pb, st)) ||
      (e = gemm(m, m->pa, (int64_t)H * B, m->pb, (int64_t)n * B, m->dw1,
                (int64_t)H * n, n, nullptr, 0, H, n, B, 0, st)))
    return cuda_check(e, "mlp dW1");
  k_colsum<<<dim3((n + 127) / 128, I), 128, 0, st>>>(m->dz2, B, n, m->db2);
  k_colsum<<<dim3((H + 127) / 128, I), 128, 0, st>>>(m->da1, B, H, m->db1);
  return cuda_check(cudaSuccess, "mlp backward");
}

int pysa_gb_mlp_adam(const pysa_gb_mlp* m, float lr, float beta1, float beta2,
                     float eps, int32_t step, void* stream) {
  if (!mlp_ok(m) || step < 1) return mlp_fail("mlp adam: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t I = m->num_instances, n = m->n, H = m->hidden;
  const float c1 = 1.0f - powf(beta1, (float)step);
  const float c2 = 1.0f - powf(beta2, (float)step);
  k_adam<<<grid_for(I * H * n), 256, 0, st>>>(m->w1, m->m1, m->v1, m->dw1,
                                               I * H * n, lr, beta1, beta2, eps,
                                               c1, c2);
  k_adam<<<grid_for(I * n * H), 256, 0, st>>>(m->w2, m->m2, m->v2, m->dw2,
                                               I * n * H, lr, beta1, beta2, eps,
                                               c1, c2);
  k_adam<<<grid_for(I * H), 256, 0, st>>>(m->b1, m->mb1, m->vb1, m->db1, I * H,
                                           lr, beta1, beta2, eps, c1, c2);
  k_adam<<<grid_for(I * n), 256, 0, st>>>(m->b2, m->mb2, m->vb2, m->db2, I * n,
                                           lr, beta1, beta2, eps, c1, c2);
  return cuda_check(mlp_repack(m, st), "mlp adam");
}

int pysa_gb_mlp_pairs(const pysa_gb_mlp* m, int32_t problem_type,
                      const int32_t* n_inst, const uint32_t* snap_a,
                      const uint32_t* snap_b, int32_t words, float* target,
                      void* stream) {
  if (!mlp_ok(m) || !snap_a || !snap_b || !target || !n_inst)
    return mlp_fail("mlp pairs: bad argument");
  k_pairs<<<dim3(grid_for((int64_t)m->batch * m->n), m->num_instances), 256,
            0, (cudaStream_t)stream>>>(snap_a, snap_b, words, n_inst,
                                       m->batch, m->n, problem_type, m->x,
                                       target);
  return cuda_check(cudaSuccess, "mlp pairs");
}

int pysa_gb_cold_rows(const pysa_gb_problems* p, const pysa_gb_state* s,
                      const int32_t* enabled, int32_t batch, int32_t* rows,
                      void* stream) {
  if (!p || !s || !rows || batch <= 0 || p->num_instances <= 0)
    return mlp_fail("cold rows: bad argument");
  k_cold_rows<<<dim3((batch + 127) / 128, p->num_instances), 128, 0,
                (cudaStream_t)stream>>>(*p, s->chain_beta, enabled, batch,
                                        rows);
  return cuda_check(cudaSuccess, "cold rows");
}

int pysa_gb_snapshot(const pysa_gb_problems* p, const pysa_gb_state* s,
                     const int32_t* rows, int32_t batch, uint32_t* out,
                     void* stream) {
  if (!p || !s || !rows || !out || batch <= 0 || p->num_instances <= 0)
    return mlp_fail("snapshot: bad argument");
  k_snapshot<<<grid_for((int64_t)p->num_instances * batch * p->words), 256, 0,
               (cudaStream_t)stream>>>(s->spins, p->words, rows, batch,
                                       p->num_instances, out);
  return cuda_check(cudaSuccess, "snapshot");
}

int64_t pysa_gb_proposal_j_elems(int32_t num_instances, int32_t nn,
                                 int32_t terms) {
  if (num_instances <= 0 || nn <= 0 || nn % 256 || terms < 1 || terms > 2)
    return mlp_fail("proposal couplings: bad size");
  return (int64_t)num_instances * terms * nn * nn;
}

int pysa_gb_pack_proposal_j(const pysa_gb_problems* p,
                            const pysa_gb_host_tables* host, int32_t nn,
                            int32_t terms, uint16_t* out, void* stream) {
  if (!p || !host || !out || nn <= 0 || nn % 256 || terms < 1 || terms > 2 ||
      p->max_n > nn)
    return mlp_fail("pack proposal couplings: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  for (int i = 0; i < p->num_instances; ++i)
    for (int t = 0; t < terms; ++t)
      k_pack_proposal_j<<<grid_for((int64_t)nn * nn), 256, 0, st>>>(
          p->J + host->j_off[i], host->n[i], host->ld[i], nn, t,
          out + ((int64_t)i * terms + t) * nn * nn);
  return cuda_check(cudaSuccess, "pack proposal couplings");
}

int pysa_gb_propose(const pysa_gb_problems* p, pysa_gb_state* s,
                    pysa_gb_workspace* ws, const pysa_gb_mlp* m,
                    const int32_t* rows, const uint16_t* j_packed,
                    int32_t terms, const pysa_gb_proposal_scratch* sc,
                    uint64_t seed, uint32_t round, float target_flips,
                    int32_t* accepted, void* stream) {
  if (!p || !s || !ws || !mlp_ok(m) || !rows || !j_packed || !sc ||
      !accepted || terms < 1 || terms > 2)
    return mlp_fail("propose: bad argument");
  if (p->num_instances != m->num_instances || p->max_n > m->n)
    return mlp_fail("propose: network does not match the problems");
  cudaStream_t st = (cudaStream_t)stream;
  const int B = m->batch, n = m->n, I = m->num_instances;
  const int64_t jn = (int64_t)n * n;
  cudaError_t e;
  k_gather_rows<<<dim3(grid_for((int64_t)B * n), I), 256, 0, st>>>(
      *p, s->spins, rows, B, n, m->x);
  if ((e = mlp_forward(m, st))) return cuda_check(e, "propose forward");
  k_sample_flips<<<dim3((B + 7) / 8, I), 256, 0, st>>>(
      *p, rows, B, n, m->z2, m->x, sc->flip, sc->delta, sc->logq_fwd, seed,
      round, target_flips);
  if ((e = mlp_forward(m, st))) return cuda_check(e, "propose reverse");
  k_logq_reverse<<<dim3((B + 7) / 8, I), 256, 0, st>>>(
      rows, B, n, p->n, m->z2, sc->flip, sc->logq_rev, target_flips);
  // jd = delta J_field^T: M = B, N = nn, K = nn; terms accumulate
  if ((e = pack(m, sc->delta, n, (int64_t)B * n, B, n, 0, 128, m->pa, st)))
    return cuda_check(e, "propose J delta");
  for (int t = 0; t < terms; ++t) {
    GemmArgs g;
    g.A = m->pa;
    g.B = j_packed + t * jn;
    g.C = sc->jd;
    g.bias = nullptr;
    g.status = m->status;
    g.strideA = (int64_t)B * n;
    g.strideB = terms * jn;
    g.strideC = (int64_t)B * n;
    g.strideBias = 0;
    g.M = B;
    g.N = n;
    g.K = n;
    g.ldc = n;
    g.accumulate = t > 0;
    g.relu = 0;
    if ((e = launch_gemm_tc(g, I, st))) return cuda_check(e, "propose J delta");
  }
  k_mh_accept<<<dim3((B + 7) / 8, I), 256, 0, st>>>(
      *p, *s, ws->fields, ws->field_ld, rows, B, n, m->x, sc->delta, sc->jd,
      sc->logq_fwd, sc->logq_rev, seed, round, accepted, sc->de);
  return cuda_check(cudaSuccess, "propose");
}

}  // extern "C"
