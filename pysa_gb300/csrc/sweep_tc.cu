// sweep_tc.cu -- blocked delayed-update Metropolis sweep on the tensor cores
// (tcgen05 + tensor memory, sm_103a).
//
// Same sweep as pysa/simulation.py:60-76 with the rule of pysa/ising.py:40-63 /
// pysa/qubo.py:40-63, sequential order, but the spins are resolved 64 at a
// time:
//   * the local fields H of the CTA's chains live in TENSOR MEMORY as an FP32
//     accumulator: TMEM lane m holds chain c = m % CC, columns of slice
//     q = m / CC (the n columns are folded into F slices of S <= 512);
//   * for a block of 64 spins each chain's thread reads its 64 fields
//     (tcgen05.ld), decides the 64 spins one after another, applying the exact
//     in-block field corrections from the FP32 64x64 diagonal block of J, and
//     writes its flips delta in {0, +-1, +-2} (exact in BF16 and E4M3) into
//     the A tile;
//   * one thread issues the cross-block update H += A * B as tcgen05.mma with
//     B = J rows of the block split as J_hi + J_lo in BF16 (one term when J is
//     exactly BF16; optionally one E4M3 term when J is exactly E4M3, the
//     E8 variants in sweep_tc_e8.cu), FP32 accumulation in TMEM.  The MMA of
//     the tile holding the next block's columns is committed first so the
//     next decisions start while the remaining tiles run.
// B tiles (pre-laid-out in the canonical no-swizzle K-major core-matrix order)
// and the diagonal blocks stream in through a ring of shared-memory stages by
// 1-D bulk copies (TMA engine).  Integer couplings make every product and sum
// exact, so trajectories match the plain sweep bit for bit.
//
// Roles: warps 0-3 decide (thread = TMEM lane; with F > 1 only the warps of
// the slice holding the block's columns, the others help: at F = 2 they
// compute the older sub-blocks' corrections and write A rows, at F = 4 they
// write A rows; in block rounds at F = 2 all four decide, two lanes per
// chain, from fields the holding slice stashes in shared memory), warp 4
// issues MMAs, warp 5 produces stages, warps 6-7 precompute the next
// block's log-uniforms.  Every wait is bounded; a
// timeout sets the status word and an abort flag that releases every other
// wait.
#include <cuda_fp8.h>

#include "aux.cuh"
#include "tc_api.h"
#include "tc_ptx.cuh"

namespace pysa_gb {

// B tile width: columns of one tile (one ring stage, one MMA group of N =
// kTW).
constexpr int kTW = 256;

// Decision mode of a block: block rounds (D64) while the previous block's
// largest flip count of any chain was at most TcArgs::round_limit (default
// 12), else sequential sub-blocks.  A round costs about as much as 6-10
// sequential spins, so the rounds win while flips are rare.

// RND: random visiting order (one permutation per instance and sweep); the
// B ring keeps two stages to make room for the gathered block fields.
// E8: operands in FP8 E4M3 (couplings exact in E4M3; deltas 0, +-1, +-2):
// half the bytes per row, so twice the ring stages in the same space.
template <int F, bool RND = false, bool E8 = false>
struct TcCfg {
  static constexpr int CC = 128 / F;          // chains per CTA
  static constexpr int NS = E8 ? (F == 1 ? 4 : F == 2 ? 6 : 8)
                               : ((F == 1 || RND) ? 2 : 3);  // B ring stages
  static constexpr int WORDS = 16 * F;        // spin words per chain
  // operand rows: K = 64 elements = ROW_B bytes, in 16-byte chunks of the
  // canonical no-swizzle K-major layout: core matrices of 8 rows x 16
  // bytes, K-adjacent ones 128 bytes apart, 8-row groups SBO bytes apart
  static constexpr int ROW_B = E8 ? 64 : 128;
  static constexpr int CPR = ROW_B / 16;      // chunks per row
  static constexpr uint32_t SBO = 8u * ROW_B;
  // A operand: ONE copy of the CC chains' delta rows (physical rows
  // 128 - CC ... 127) with 128 - CC zero rows on either side; slice q's
  // 128-row MMA operand starts (128 - CC - q CC) rows in, so only its own
  // chains' rows fall on its lanes.
  // fold 4: two A buffers (block t writes buffer t & 1 while the MMAs of
  // block t - 1 still read the other), interleaved with the zero rows:
  // [zero][buffer 0][zero][buffer 1][zero]; buffer b's delta rows are
  // 128 - CC + 128 b ...
  static constexpr int A_NBUF = F == 4 ? 2 : 1;
  static constexpr int A_ROWS =
      F == 1 ? 128 : (A_NBUF == 2 ? 384 - CC : 256 - CC);
  static constexpr size_t A_OFF = 0;
  static constexpr size_t A_BYTES = (size_t)A_ROWS * ROW_B;
  static constexpr size_t B_OFF = A_OFF + A_BYTES;
  static constexpr size_t B_STAGE = (size_t)kTW * ROW_B;  // one tile
  static constexpr size_t JBB_OFF = B_OFF + NS * B_STAGE;
  static constexpr size_t SPIN_OFF = JBB_OFF + 2 * 16384;
  // log-uniforms of a block: two buffers of [chain][64] floats in the
  // swizzled order of cidx() (16-byte stores and loads without bank
  // conflicts)
  static constexpr size_t LF_OFF = SPIN_OFF + (size_t)CC * WORDS * 4;
  static constexpr size_t DL_OFF = LF_OFF + (size_t)2 * 64 * CC * 4;
  // deltas [64][CC] (sequential sub-blocks) or the block's loaded fields
  // [chain][64] swizzled (block rounds)
  static constexpr size_t DE_OFF = DL_OFF + (size_t)64 * CC * 4;
  static constexpr size_t E0_OFF = DE_OFF + (size_t)CC * 8;
  static constexpr size_t EPART_OFF = E0_OFF + (size_t)CC * 8;
  static constexpr size_t BETA_OFF = EPART_OFF + (size_t)F * CC * 8;
  // F == 2: corrections of sub-blocks 2 and 3 from the older sub-blocks,
  // computed by the idle slice's threads ([2][16][CC] floats)
  static constexpr bool HELP = F == 2;
  // F == 4: the three idle slices' warps write the A rows of sub-blocks 0-2
  static constexpr bool APUT = F == 4;
  // F == 2, visiting order: block rounds run on all four decision warps,
  // two lanes per chain (the other slice's warps would idle)
  static constexpr bool PAIRS = F == 2 && !RND;
  // 1 / (beta scale) of each chain (+inf for beta <= 0), kept with beta_s
  static constexpr size_t INVB_OFF = BETA_OFF + CC * 4;
  static constexpr size_t CORR_OFF = INVB_OFF + CC * 4;
  static constexpr size_t CORR_BYTES = HELP ? (size_t)2 * 16 * CC * 4 : 0;
  // RND, F > 1: fields of the block's 64 scattered columns, gathered by the
  // warps whose slices hold them ([64][CC] floats)
  static constexpr size_t HBUF_OFF = CORR_OFF + CORR_BYTES;
  static constexpr size_t HBUF_BYTES =
      (RND && F > 1) ? (size_t)64 * CC * 4 : 0;
  // RND: each decision warp's copy of the block's 64 permutation entries
  static constexpr size_t PERM_OFF = HBUF_OFF + HBUF_BYTES;
  static constexpr size_t PERM_BYTES = RND ? (size_t)4 * 64 * 4 : 0;
  // RND: position-ordered spin words of the next blocks, [2][2][CC], made
  // by the log-uniform helper warps
  static constexpr size_t POSB_OFF = PERM_OFF + PERM_BYTES;
  static constexpr size_t POSB_BYTES = RND ? (size_t)2 * 2 * CC * 4 : 0;
  static constexpr size_t BAR_OFF = (POSB_OFF + POSB_BYTES + 63) / 64 * 64;
  // a_full, mma_done, h_ready, jbb_full[2], jbb_free[2], rc_full, rc_done,
  // lf_full[2], lf_free[2], full[NS], free[NS], drain, mma_done_b[2]
  static constexpr int NBARS = 16 + 2 * NS;
  static constexpr size_t MISC_OFF = BAR_OFF + NBARS * 8;
  // tmem slot, abort flag, current unit (item, first sweep, sweeps), then
  // per block parity and decision warp the block's largest flip count of a
  // chain ([2][4] int32)
  static constexpr size_t STAT_OFF = MISC_OFF + 32;
  static constexpr size_t BYTES = STAT_OFF + 32;
  static_assert(BYTES <= 232448, "shared memory budget");
};

struct TcShared {
  uint64_t *a_full, *mma_done, *h_ready, *jbb_full, *jbb_free, *rc_full,
      *rc_done, *lf_full, *lf_free, *full, *free_, *drain, *mma_done_b;
  uint32_t* tmem_slot;
  volatile int32_t* abort;
};

__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity,
                                        const TcShared& sh, int32_t* status) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*sh.abort) return false;
    if (globaltimer_ns() - t0 > 1000000000ull) {
      set_status(status, PYSA_GB_ERR_TIMEOUT);
      *sh.abort = 1;
      return false;
    }
  }
}

// After an abort: wait (bounded, about a second, whatever the abort flag
// says) for a barrier phase that only asynchronous work already issued by
// this CTA completes -- bulk copies landing in shared memory, MMAs writing
// tensor memory -- so that none is in flight when the CTA frees its tensor
// memory and exits.
__device__ __forceinline__ void drain_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return;
  const uint64_t t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity))
    if (globaltimer_ns() - t0 > 1000000000ull) return;
}

// Every MMA up to and including block Gx has completed.  One A buffer: the
// per-block barrier, at most one phase behind (each block waits for its
// predecessor's MMAs before writing A).  Two A buffers (fold 4): blocks Gx
// and Gx - 1 may both be pending, and a parity wait on the per-block
// barrier cannot tell their phases apart, so the per-buffer barriers are
// waited instead (their latest phases are these blocks').
template <int NBUF>
__device__ __forceinline__ bool mmas_done_through(uint32_t Gx,
                                                  const TcShared& sh,
                                                  int32_t* status) {
  if (NBUF == 1) return tc_wait(sh.mma_done, Gx & 1, sh, status);
  if (!tc_wait(&sh.mma_done_b[Gx & 1], (Gx >> 1) & 1, sh, status))
    return false;
  return Gx == 0 || tc_wait(&sh.mma_done_b[(Gx - 1) & 1],
                            ((Gx - 1) >> 1) & 1, sh, status);
}

// (sum, compensation) + x with Neumaier's compensated summation in f32
__device__ __forceinline__ float2 add_compensated(float2 acc, float x) {
  const float t = acc.x + x;
  const float e = fabsf(acc.x) >= fabsf(x) ? (acc.x - t) + x : (x - t) + acc.x;
  return make_float2(t, acc.y + e);
}

// Timeline stamps (SM clock cycles) of CTA 0 when a trace buffer is given,
// in builds with
// PYSA_GB_TRACE defined (diagnostics only: the stamps' branches in the
// decision loop cost about 8 % of a sweep, so release builds drop them):
// row G < 48 per block, row 48 whole-unit marks (entry, set-up done, last
// MMA done, fields stored, unit done, field load start; the last unit's).
__device__ __forceinline__ void stamp(const TcArgs& a, uint32_t G, int slot) {
#ifdef PYSA_GB_TRACE
  if (a.trace && blockIdx.x == 0 && G < 48)
    a.trace[G * 24 + slot] = clock64();
#endif
}
// Trace builds: counters of CTA 0 in row 48, slots 8 + i (i = 0: blocks
// decided in rounds, 1: in sequential sub-blocks, 2: rounds).
__device__ __forceinline__ void count(const TcArgs& a, int i, long long v) {
#ifdef PYSA_GB_TRACE
  if (a.trace && blockIdx.x == 0)
    atomicAdd(reinterpret_cast<unsigned long long*>(a.trace + 48 * 24 + 8 + i),
              (unsigned long long)v);
#endif
}
__device__ __forceinline__ void stamp_cta(const TcArgs& a, int slot) {
#ifdef PYSA_GB_TRACE
  if (a.trace && blockIdx.x == 0) a.trace[48 * 24 + slot] = clock64();
#endif
}

// Named barriers in inline PTX: the warp is reconverged first and the
// non-aligned barrier.sync form is used, since the compiler does not insert
// the reconvergence it adds before __syncthreads().
__device__ __forceinline__ void named_sync_128() {
  __syncwarp();
  asm volatile("barrier.sync 1, 128;" ::: "memory");
}

// Deciding and helping threads of the four decision warps (fold 2).
__device__ __forceinline__ void named_sync_dec() {
  __syncwarp();
  asm volatile("barrier.sync 3, 128;" ::: "memory");
}
// Fold 4: the deciding warp announces sub-blocks 0-2 without waiting; the
// three other warps wait for it (the same barrier, 128 threads in all)
__device__ __forceinline__ void named_arrive_aput() {
  __syncwarp();
  asm volatile("barrier.arrive 3, 128;" ::: "memory");
}
__device__ __forceinline__ void named_sync_aput() {
  __syncwarp();
  asm volatile("barrier.sync 3, 128;" ::: "memory");
}

__device__ __forceinline__ void named_sync_helpers() {
  __syncwarp();
  asm volatile("barrier.sync 2, 64;" ::: "memory");
}

// Index of value k (< 64) of chain c in a [chain][64] array whose 16-byte
// chunks are XOR-swizzled by c % 8: a quarter-warp's 16-byte accesses to the
// same chunk of 8 consecutive chains land on 8 distinct bank groups.
__device__ __forceinline__ int cidx(int c, int k) {
  return c * 64 + ((((k >> 2) ^ (c & 7)) << 2) | (k & 3));
}

// The log-uniform buffers hold a = log u - m, m = 3e-5 + 1e-6 |log u|: the
// rejection bound in the log domain, so that the rejection threshold in
// field units is a / (beta scale) and the acceptance threshold
// min((a + 2 m') / (beta scale), 0) with m' = 3e-5 + 1e-6 |a| >= m (a slightly
// wider band: decisions outside it stay certain).  lf_of(a) = a + m' is a
// log u estimate within 1e-9 relative, well inside the margin of
// metropolis_accept_lf, for its exact rule.
__device__ __forceinline__ float lf_of(float a) {
  return a + fmaf(1e-6f, fabsf(a), 3e-5f);
}

__device__ __forceinline__ uint32_t bf16_bits(float d) {
  // exact for d in {0, +-1, +-2}
  return __float_as_uint(d) >> 16;
}

// E4M3 bits of d in {0, +-1, +-2} (exponent bias 7, three mantissa bits:
// 1 = 0x38, 2 = 0x40, sign 0x80); zero of either sign is 0.
__device__ __forceinline__ uint32_t e4m3_bits(float d) {
  const uint32_t u = __float_as_uint(d);
  if ((u & 0x7FFFFFFFu) == 0u) return 0u;
  return ((((u >> 23) & 0xFFu) - 120u) << 3) | ((u >> 24) & 0x80u);
}

// The rare exact redo of one deciding thread's sub-block (some decision of
// the warp fell inside the f32 band), kept out of line: inlined, its code
// and registers slow the fast path by about 12 %.  It rebuilds the
// sub-block's fields exactly as the fast path does (same loads, same
// correction order), decides every spin with the exact rule and writes the
// deltas to dl_s; returns the new spin word and block energy change.
struct RedoCtx {
  const float* jb;          // diagonal block of the block, [64][64]
  float* dl_s;              // deltas [64][CC]
  const float* corr_s;      // helper corrections (fold 2)
  const float* hbuf;        // gathered fields (random order, fold > 1)
  const int32_t* perm_w;    // this warp's visiting positions (random order)
  const float* lfb;         // log-uniforms [chain][64], cidx() order
  uint32_t taddr;           // TMEM address of the thread's lane
  int co, kmax, c, g, i0, sb;
  int valid, ising;
  float beta;
  uint64_t seed;
  uint32_t inst, sweep, chain_local;
  uint32_t wsave;           // spin word before the sub-block
  float dEsave;
};

template <int F, bool RND>
__device__ __noinline__ void redo_subblock(const RedoCtx& x, uint32_t* wcur,
                                           float* dEb) {
  constexpr int CC = 128 / F;
  const int g = x.g, c = x.c;
  float hs[16];
  if constexpr (!RND) {
    tc::tmem_ld16(x.taddr + x.co + 16 * g, hs);
  } else if constexpr (F > 1) {
#pragma unroll
    for (int j = 0; j < 16; ++j)
      hs[j] = 16 * g + j < x.kmax ? x.hbuf[(16 * g + j) * CC + c] : 0.0f;
  } else {
    uint32_t r[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int sp = x.perm_w[16 * g + j];
      r[j] = 0u;
      if (sp >= 0) r[j] = tc::tmem_ld1_nowait(x.taddr + (uint32_t)sp);
    }
    tc::tmem_wait_ld16(r);
#pragma unroll
    for (int j = 0; j < 16; ++j) hs[j] = __uint_as_float(r[j]);
  }
  const bool help = F == 2;
  if (help && g >= 2) {
#pragma unroll
    for (int j = 0; j < 16; ++j) hs[j] += x.corr_s[((g - 2) * 16 + j) * CC + c];
  }
  for (int k = help && g >= 2 ? 16 * (g - 1) : 0; k < 16 * g; ++k) {
    const float d = x.dl_s[k * CC + c];
    const float4* jr = reinterpret_cast<const float4*>(x.jb + k * 64 + 16 * g);
#pragma unroll
    for (int q4 = 0; q4 < 4; ++q4) {
      const float4 v = jr[q4];
      hs[4 * q4 + 0] = fmaf(d, v.x, hs[4 * q4 + 0]);
      hs[4 * q4 + 1] = fmaf(d, v.y, hs[4 * q4 + 1]);
      hs[4 * q4 + 2] = fmaf(d, v.z, hs[4 * q4 + 2]);
      hs[4 * q4 + 3] = fmaf(d, v.w, hs[4 * q4 + 3]);
    }
  }
  uint32_t w = x.wsave;
  float e = x.dEsave;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const int k = 16 * g + j;
    const bool sbit = (w >> (x.sb + j)) & 1u;
    const float hk = hs[j];
    const float dn =
        x.ising ? (sbit ? 2.0f * hk : -2.0f * hk) : (sbit ? hk : -hk);
    const bool acc = x.valid && k < x.kmax &&
                     metropolis_accept_lf(dn, x.beta, lf_of(x.lfb[cidx(c, k)]),
                                          x.seed, x.inst, x.sweep,
                                          x.chain_local, (uint32_t)(x.i0 + k));
    const float dl =
        acc ? (x.ising ? (sbit ? -2.0f : 2.0f) : (sbit ? -1.0f : 1.0f)) : 0.0f;
    x.dl_s[k * CC + c] = dl;
    if (acc) {
      e -= dn;
      w ^= 1u << (x.sb + j);
    }
    if (j < 15) {
      const float4* jr =
          reinterpret_cast<const float4*>(x.jb + k * 64 + 16 * g);
#pragma unroll
      for (int q4 = (j + 1) >> 2; q4 < 4; ++q4) {
        const float4 v = jr[q4];
        if (4 * q4 + 0 > j) hs[4 * q4 + 0] = fmaf(dl, v.x, hs[4 * q4 + 0]);
        if (4 * q4 + 1 > j) hs[4 * q4 + 1] = fmaf(dl, v.y, hs[4 * q4 + 1]);
        if (4 * q4 + 2 > j) hs[4 * q4 + 2] = fmaf(dl, v.z, hs[4 * q4 + 2]);
        if (4 * q4 + 3 > j) hs[4 * q4 + 3] = fmaf(dl, v.w, hs[4 * q4 + 3]);
      }
    }
  }
  *wcur = w;
  *dEb = e;
}

// Work units.  Fixed units (a.wrap == 0): unit u is item u % num_items for
// sweeps (u / num_items) * unit_sweeps ... + unit_sweeps - 1 of the launch,
// taken from a queue in order.  Wrap-around units (a.wrap == 1, items of one
// size, unit_sweeps = the launch's sweeps): each CTA takes a share from the
// queue and runs its pieces (wrap_piece).  Either way a unit waits (bounded)
// until its item has run the sweeps before it, which a CTA that took its
// work from the queue earlier (so is running) owns, so the wait always ends.
// Within a unit the fields stay in TMEM across sweeps; the replica exchange
// of the item's reads runs in the kernel when fused.
template <int F, bool RND, bool E8>
__global__ void __launch_bounds__(256, 1) k_sweep_tc(const TcArgs a) {
  using C = TcCfg<F, RND, E8>;
  constexpr int CC = C::CC;
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::BAR_OFF);
  TcShared sh;
  sh.a_full = bars + 0;
  sh.mma_done = bars + 1;
  sh.h_ready = bars + 2;
  sh.jbb_full = bars + 3;
  sh.jbb_free = bars + 5;
  sh.rc_full = bars + 7;
  sh.rc_done = bars + 8;
  sh.lf_full = bars + 9;
  sh.lf_free = bars + 11;
  sh.full = bars + 13;
  sh.free_ = bars + 13 + C::NS;
  sh.drain = bars + 13 + 2 * C::NS;
  sh.mma_done_b = bars + 14 + 2 * C::NS;  // [2]: MMAs of blocks using A
                                          // buffer 0 / 1 (two buffers)
  sh.tmem_slot = reinterpret_cast<uint32_t*>(smem + C::MISC_OFF);
  sh.abort = reinterpret_cast<volatile int32_t*>(smem + C::MISC_OFF + 8);
  volatile int32_t* unit_s =  // [item, first sweep, sweeps] of the unit
      reinterpret_cast<volatile int32_t*>(smem + C::MISC_OFF + 16);
  volatile uint32_t* stat_s =
      reinterpret_cast<volatile uint32_t*>(smem + C::STAT_OFF);
  uint32_t* spins_s = reinterpret_cast<uint32_t*>(smem + C::SPIN_OFF);
  double* dE_s = reinterpret_cast<double*>(smem + C::DE_OFF);
  double* e0_s = reinterpret_cast<double*>(smem + C::E0_OFF);
  double* epart_s = reinterpret_cast<double*>(smem + C::EPART_OFF);
  float* beta_s = reinterpret_cast<float*>(smem + C::BETA_OFF);
  float* invb_s = reinterpret_cast<float*>(smem + C::INVB_OFF);
  // the field-unit scale of a chain's rejection threshold: 1 / (beta scale)
  auto inv_bs = [&](float b) {
    return b > 0.0f ? 1.0f / (b * (a.p.problem_type == PYSA_GB_ISING ? 2.0f
                                                                     : 1.0f))
                    : INFINITY;
  };
  const float* jbb = reinterpret_cast<const float*>(smem + C::JBB_OFF);
  float* lf_s = reinterpret_cast<float*>(smem + C::LF_OFF);
  float* dl_s = reinterpret_cast<float*>(smem + C::DL_OFF);
  float* corr_s = reinterpret_cast<float*>(smem + C::CORR_OFF);
  float* hbuf = reinterpret_cast<float*>(smem + C::HBUF_OFF);
  int32_t* perm_s = reinterpret_cast<int32_t*>(smem + C::PERM_OFF);
  uint32_t* posb = reinterpret_cast<uint32_t*>(smem + C::POSB_OFF);
  // exchange scratch between sweeps (dl_s is idle then): energies [CC],
  // per warp slot->replica, uniforms, their logs and the betas [4][CC] each
  float* ex_E = dl_s;
  int32_t* ex_B = reinterpret_cast<int32_t*>(dl_s + CC);
  uint32_t* ex_X = reinterpret_cast<uint32_t*>(dl_s + 5 * CC);
  float* ex_L = dl_s + 9 * CC;
  float* ex_T = dl_s + 13 * CC;
  // per pair k: the lower slot's replica before the pass, its energy and the
  // betas' difference ([4][CC] each)
  int32_t* ex_B2 = reinterpret_cast<int32_t*>(dl_s + 17 * CC);
  float* ex_E2 = dl_s + 21 * CC;
  float* ex_D = dl_s + 25 * CC;
  const uint32_t smem_base = smem_addr(smem);
  // A operand: physical row m, and the element of position j (< 64) of a
  // row set to +-1 (QUBO) or +-2 (Ising) deltas
  auto a_row = [&](int m) {
    return smem + C::A_OFF + ((m >> 3) * C::CPR) * 128 + (m & 7) * 16;
  };
  const bool ising = a.p.problem_type == PYSA_GB_ISING;
  auto a_put = [&](unsigned char* rowp, int j, bool neg) {
    if constexpr (E8)
      rowp[(j >> 4) * 128 + (j & 15)] =
          (unsigned char)((ising ? 0x40u : 0x38u) | (neg ? 0x80u : 0u));
    else
      *reinterpret_cast<uint16_t*>(rowp + (j >> 3) * 128 + (j & 7) * 2) =
          (uint16_t)((ising ? 0x4000u : 0x3F80u) | (neg ? 0x8000u : 0u));
  };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t* status = a.s.status;
  const uint32_t sweep0 = (uint32_t)(*a.s.sweep_counter);
  const int total_units = a.num_items * a.units_per_item;
  const int T = a.terms;
  constexpr uint32_t kCols = 512;

  // ---------------------------------------------------------------- set-up
  if (threadIdx.x == 0) stamp_cta(a, 0);
  if (warp == 0) {
    tc::tmem_alloc(sh.tmem_slot, kCols);
    tc::tmem_relinquish();
  }
  if (threadIdx.x == 32) {
    for (int b = 0; b < C::NBARS; ++b) mbar_init(&bars[b], 1);
    *sh.abort = 0;
    fence_mbar_init();
  }
  for (int i = threadIdx.x; i < (int)(C::A_BYTES / 16); i += blockDim.x)
    reinterpret_cast<uint4*>(smem + C::A_OFF)[i] = make_uint4(0, 0, 0, 0);
  fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *sh.tmem_slot;
  const uint32_t idesc_full =
      E8 ? tc::idesc_e4m3(128, kTW) : tc::idesc_bf16(128, kTW);

  // decision-thread identity: TMEM lane L = slice q, chain c
  const int L = threadIdx.x;
  const int q = L / CC, c = L % CC;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  float* stg = reinterpret_cast<float*>(smem + C::B_OFF) + warp * (32 * 33);
  const int w_c0 = (32 * warp) % CC, w_q = (32 * warp) / CC;

  // per-role running counters (identical sequences in every role)
  uint32_t G = 0;   // blocks
  uint32_t RG = 0;  // recompute blocks
  uint32_t u = 0;   // B ring stages (producer and MMA)
  // decision warps: this block's decision mode (the same in all 128 threads);
  // sequential until a block shows few flips
  bool d64 = a.decision_mode == 1;
  int share = -1, piece = 0;  // thread 0, wrap-around units

  for (;;) {
    // ------------------------------------------------------ next unit
    if (threadIdx.x == 0) {
      int it = -1, sb = 0, sl = 0;
      if (!*sh.abort) {
        if (a.wrap) {
          if (share < 0)
            share = (int)atomicAdd(reinterpret_cast<unsigned*>(a.sched), 1u);
          if (!wrap_piece(a.num_items, a.unit_sweeps, (int)gridDim.x, share,
                          piece++, &it, &sb, &sl))
            it = -1;
        } else {
          const int un =
              (int)atomicAdd(reinterpret_cast<unsigned*>(a.sched), 1u);
          if (un < total_units) {
            it = un % a.num_items;
            sb = (un / a.num_items) * a.unit_sweeps;
            sl = a.unit_sweeps;
          }
        }
        if (it >= 0) {
          volatile int32_t* done = a.sched + 2 + it;  // sweeps run
          if (*done < sb) {
            const uint64_t lim =
                a.unit_wait_ns ? a.unit_wait_ns : 1000000000ull;
            const uint64_t t0 = globaltimer_ns();
            while (*done < sb) {
              if (globaltimer_ns() - t0 > lim) {
                set_status(status, PYSA_GB_ERR_TIMEOUT);
                *sh.abort = 1;
                it = -1;
                break;
              }
            }
          }
          __threadfence();  // the previous unit's stores are visible
        }
      }
      unit_s[0] = it;
      unit_s[1] = sb;
      unit_s[2] = sl;
    }
    __syncthreads();
    const int un_item = unit_s[0];
    if (un_item < 0) break;
    const int un_first = unit_s[1];
    const int KU = unit_s[2];
    const TcItem item = a.items[un_item];
    const uint32_t sweep_first = sweep0 + (uint32_t)un_first;
    const int inst = item.inst;
    const int n = a.p.n[inst];
    const int NP = (n + 64 * F - 1) / (64 * F) * (64 * F);
    const int S = NP / F;
    const int NB = (n + 63) / 64;
    const int NT = (S + kTW - 1) / kTW;
    const int words = (n + 31) >> 5;
    const int64_t chain_base = a.p.chain_off[inst];
    const bool valid = warp < 4 && c < item.nchains;
    const int64_t chain = item.chain0 + c;
    const uint32_t chain_local = (uint32_t)(chain - chain_base);
    const uint32_t G0 = G, RG0 = RG;
    const uint32_t Gend = G0 + (uint32_t)(KU * NB);
    auto rc_at = [&](int s) {
      return a.recompute_every > 0 &&
             ((sweep_first + (uint32_t)s) % (uint32_t)a.recompute_every) == 0;
    };
    int n_rc = 0;
    for (int s = 0; s < KU; ++s) n_rc += rc_at(s) ? 1 : 0;
    // producer lane: ring stages issued before this unit, last diagonal
    // block issued in it (for the drain after an abort)
    const uint32_t u_first = u;
    uint32_t jbb_last = 0xFFFFFFFFu;

    // ------------------------------------------------ unit prologue
    for (int i = threadIdx.x; i < CC * C::WORDS; i += blockDim.x) {
      const int w = i / CC, cc = i % CC;  // layout [word][chain]
      spins_s[i] = (cc < item.nchains && w < words)
                       ? __ldcg(a.s.spins + (item.chain0 + cc) * (int64_t)a.p.words + w)
                       : 0u;
    }
    for (int cc = threadIdx.x; cc < CC; cc += blockDim.x) {
      dE_s[cc] = 0.0;
      // state written by other CTAs of this launch: loads bypass L1
      e0_s[cc] = cc < item.nchains
                     ? (double)__ldcg(a.s.energies + item.chain0 + cc)
                     : 0.0;
      beta_s[cc] =
          cc < item.nchains ? __ldcg(a.s.chain_beta + item.chain0 + cc) : 0.0f;
      invb_s[cc] = inv_bs(beta_s[cc]);
    }
    if (threadIdx.x == 0) stamp_cta(a, 5);
    if (warp < 4 && !rc_at(0)) {  // local fields -> TMEM
      // two 32-column chunks per round: 16 independent 16-byte loads in
      // flight; rows move through a per-warp shared-memory transpose (in
      // the B ring, idle until the producer starts)
      auto load4 = [&](int j0, int it) {
        const int col = w_q * S + j0 + 4 * (lane & 7);
        const int cr = w_c0 + 4 * it + (lane >> 3);
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (j0 < S && cr < item.nchains) {
          const float* f =
              a.fields + (item.chain0 + cr) * (int64_t)a.field_ld + col;
          if (col + 4 <= n) {
            v = __ldcg(reinterpret_cast<const float4*>(f));
          } else {
            v.x = col < n ? __ldcg(f) : 0.0f;
            v.y = col + 1 < n ? __ldcg(f + 1) : 0.0f;
            v.z = col + 2 < n ? __ldcg(f + 2) : 0.0f;
          }
        }
        return v;
      };
      for (int j0 = 0; j0 < S; j0 += 64) {
        float4 va[8], vb[8];
#pragma unroll
        for (int it = 0; it < 8; ++it) {
          va[it] = load4(j0, it);
          vb[it] = load4(j0 + 32, it);
        }
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
#pragma unroll
          for (int it = 0; it < 8; ++it) {
            const float4 v = h2 ? vb[it] : va[it];
            float* d = stg + (4 * it + (lane >> 3)) * 33 + 4 * (lane & 7);
            d[0] = v.x;
            d[1] = v.y;
            d[2] = v.z;
            d[3] = v.w;
          }
          __syncwarp();
          float v[32];
#pragma unroll
          for (int i = 0; i < 32; ++i) v[i] = stg[lane * 33 + i];
          __syncwarp();
          tc::tmem_st32(taddr + lane_base + j0 + 32 * h2, v);
        }
      }
      tc::tmem_wait_st();
    }
    fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x == 0) stamp_cta(a, 1);

    if (warp < 4) {
      for (int s = 0; s < KU; ++s) {
        const uint32_t sweep = sweep_first + (uint32_t)s;
        const uint32_t Gs = G0 + (uint32_t)(s * NB);  // first block of sweep
        if (rc_at(s)) {
          // ========================================== recompute: A = spins
          // the previous sweep's MMAs (which read A) must be done
          bool rok = true;
          if (s > 0) rok = mmas_done_through<C::A_NBUF>(Gs - 1, sh, status);
          for (int t = 0; t < NB; ++t) {
            const uint32_t R_ = RG + (uint32_t)t;
            bool go = rok && q == 0 && !*sh.abort;
            if (go && t > 0) go = tc_wait(sh.rc_done, (R_ - 1) & 1, sh, status);
            go = __all_sync(0xffffffffu, go);
            if (go) {
              const uint32_t w0 = spins_s[(2 * t) * CC + c];
              const uint32_t w1 = spins_s[(2 * t + 1) * CC + c];
              const int kmax = n - 64 * t < 64 ? n - 64 * t : 64;
              uint32_t pk[C::ROW_B / 4];
#pragma unroll
              for (int k = 0; k < 64; ++k) {
                const bool sb =
                    k < 32 ? ((w0 >> k) & 1u) : ((w1 >> (k - 32)) & 1u);
                const float v = (!valid || k >= kmax) ? 0.0f
                                : sb ? 1.0f : (ising ? -1.0f : 0.0f);
                if constexpr (E8) {
                  const uint32_t b8 = e4m3_bits(v) << (8 * (k & 3));
                  if (k & 3) pk[k >> 2] |= b8; else pk[k >> 2] = b8;
                } else {
                  const uint32_t b16 = bf16_bits(v);
                  if (k & 1) pk[k >> 1] |= b16 << 16; else pk[k >> 1] = b16;
                }
              }
              {
                unsigned char* rowp = a_row(128 - CC + c);  // chain c's row
#pragma unroll
                for (int kc = 0; kc < C::CPR; ++kc)
                  *reinterpret_cast<uint4*>(rowp + kc * 128) =
                      make_uint4(pk[4 * kc], pk[4 * kc + 1], pk[4 * kc + 2],
                                 pk[4 * kc + 3]);
              }
              fence_proxy_async();
            }
            named_sync_128();
            if (threadIdx.x == 0) mbar_arrive(sh.rc_full);
          }
          if (!*sh.abort && NB > 0)
            tc_wait(sh.rc_done, (RG + NB - 1) & 1, sh, status);
          RG += NB;
          tc::fence_after_sync();
          // H = J s + h in TMEM; energies sum_j s_j ((J s)_j / 2 + h_j)
          const float* hh = a.p.h + a.p.h_off[inst];
          // energy terms s_j (v_j / 2 + h_j), each split exactly into two
          // f32 parts and summed with Neumaier's compensation: f64
          // accuracy from the FP32 pipe
          float2 ep = make_float2(0.0f, 0.0f);
          if (__all_sync(0xffffffffu, !*sh.abort)) {
            for (int j0 = 0; j0 < S; j0 += 32) {
              float v[32];
              tc::tmem_ld32(taddr + lane_base + j0, v);
#pragma unroll
              for (int i = 0; i < 32; ++i) {
                const int col = q * S + j0 + i;
                if (col < n) {
                  const uint32_t wv = spins_s[(col >> 5) * CC + c];
                  const float sj =
                      ((wv >> (col & 31)) & 1u) ? 1.0f : (ising ? -1.0f : 0.0f);
                  const float hj = hh[col];
                  const float hv = 0.5f * v[i];  // exact
                  const float hi = hv + hj;
                  const float bp = hi - hv;
                  const float lo = (hv - (hi - bp)) + (hj - bp);  // hv+hj-hi
                  ep = add_compensated(ep, sj * hi);
                  ep.y += sj * lo;
                  v[i] = v[i] + hj;
                }
              }
              tc::tmem_st32(taddr + lane_base + j0, v);
            }
            tc::tmem_wait_st();
          }
          epart_s[q * CC + c] = (double)ep.x + (double)ep.y;
          tc::fence_before_sync();
          named_sync_128();
          tc::fence_after_sync();
          if (q == 0 && valid) {
            double e = 0.0;
            for (int qq = 0; qq < F; ++qq) e += epart_s[qq * CC + c];
            // drift check: the energy the sweeps accumulated against the one
            // just rebuilt from the spins (not at sweep 0, whose energies
            // may be the caller's own)
            const double acc_e = e0_s[c] + dE_s[c];
            if (sweep > 0 && !(fabs(acc_e - e) <= 1e-3 * fmax(1.0, fabs(e))))
              set_status(status, PYSA_GB_ERR_DRIFT);
            e0_s[c] = (double)(float)e;
            dE_s[c] = 0.0;
          }
          named_sync_128();
        }

        // ============================================================ decide
        const float beta = beta_s[c];
        // random order: this sweep's permutation (position -> spin)
        const int32_t* pi_row =
            RND ? a.perm + ((int64_t)(sweep % (uint32_t)a.perm_slots) *
                                a.p.num_instances + inst) * a.p.max_n
                : nullptr;
        for (int t = 0; t < NB; ++t) {
          const uint32_t Gb = Gs + (uint32_t)t;
          const int i0 = 64 * t;
          // deciding slice: the one holding the block's columns, or slice 0
          // in random order (columns scattered over all slices)
          const int qt = RND ? 0 : i0 / S, co = i0 % S;
          const int kmax = n - i0 < 64 ? n - i0 : 64;
          const bool wait_h = Gb > G0 && !(t == 0 && rc_at(s));
          // random order: lane l holds the spins at positions l and 32 + l
          // of this block (-1 past the end) with their slice and column;
          // everything else reads them by warp shuffle
          int pk0 = -1, pk1 = -1, ps0 = -1, ps1 = -1, pc0 = 0, pc1 = 0;
          if constexpr (RND) {
            if (warp < 4) {
              if (lane < kmax) pk0 = pi_row[i0 + lane];
              if (32 + lane < kmax) pk1 = pi_row[i0 + 32 + lane];
              if (pk0 >= 0) { ps0 = pk0 / S; pc0 = pk0 - ps0 * S; }
              if (pk1 >= 0) { ps1 = pk1 / S; pc1 = pk1 - ps1 * S; }
              perm_s[warp * 64 + lane] = pk0;
              perm_s[warp * 64 + 32 + lane] = pk1;
              __syncwarp();
            }
          }
          // spin at position k of this block (-1 past the end), from this
          // warp's copy (same address in every lane: a broadcast load)
          auto spos = [&](int k) { return perm_s[warp * 64 + k]; };
          if constexpr (RND && F > 1) {
            // every decision warp copies the block's fields held in its own
            // slice (TMEM lanes belong to warps) into hbuf[k][chain]
            bool hok = !*sh.abort;
            if (hok && wait_h)
              hok = tc_wait(sh.h_ready, (Gb - 1) & 1, sh, status);
            hok = __all_sync(0xffffffffu, hok);
            if (hok) {
              tc::fence_after_sync();
              for (int k0 = 0; k0 < 64; k0 += 16) {
                uint32_t r[16];
                int mine = 0;  // bit kk: position k0 + kk lives in my slice
#pragma unroll
                for (int kk = 0; kk < 16; ++kk) {
                  const int k = k0 + kk;
                  const int sl =
                      __shfl_sync(0xffffffffu, k < 32 ? ps0 : ps1, k & 31);
                  const int col =
                      __shfl_sync(0xffffffffu, k < 32 ? pc0 : pc1, k & 31);
                  r[kk] = 0u;
                  if (sl == q) {
                    r[kk] = tc::tmem_ld1_nowait(taddr + lane_base +
                                                (uint32_t)col);
                    mine |= 1 << kk;
                  }
                }
                tc::tmem_wait_ld();
#pragma unroll
                for (int kk = 0; kk < 16; ++kk)
                  if ((mine >> kk) & 1)
                    hbuf[(k0 + kk) * CC + c] = __uint_as_float(r[kk]);
              }
            }
            named_sync_128();
          }
          uint32_t blk_mf = 0u;  // largest flip count of a chain (deciders)
          if (C::PAIRS && d64) {
            // ------------------- block rounds on the four decision warps
            // The slice holding the block loads its 64 fields from TMEM into
            // dl_s ([chain][64], swizzled); then every chain is decided by
            // two lanes of one warp: lane (cc, hf), cc = 16 warp + lane % 16,
            // hf = lane / 16, tests positions 32 hf .. 32 hf + 31, its
            // partner is lane ^ 16.  Each round both lanes take the chain's
            // first candidate over all 64 positions (the partner's mask by
            // shuffle) and decide it identically; an accepted flip corrects
            // each lane's half of the fields.  The decisions, and every
            // rounding on their way, are those of the one-lane rounds below.
            // Chains by groups of 8 (a quarter-warp's 16-byte accesses stay
            // on distinct bank groups): warp w holds groups w and 7 - w, so
            // replicas that start at neighbouring temperatures (and flip
            // alike while the ladder has not mixed them) spread over the
            // warps instead of loading one of them.
            const int hf = lane >> 4;
            const int cc =
                8 * (((lane >> 3) & 1) ? 7 - warp : warp) + (lane & 7);
            bool ok = !*sh.abort;
            if (ok && q == qt && wait_h)
              ok = tc_wait(sh.h_ready, (Gb - 1) & 1, sh, status);
            if (ok) ok = tc_wait(&sh.jbb_full[Gb & 1], (Gb >> 1) & 1, sh, status);
            if (ok) ok = tc_wait(&sh.lf_full[Gb & 1], (Gb >> 1) & 1, sh, status);
            ok = __all_sync(0xffffffffu, ok);
            if (L == 0) stamp(a, Gb, 0);
            if (L == 0) stamp(a, Gb, 1);
            if (ok && q == qt) {
              tc::fence_after_sync();
              float hl[64];
              tc::tmem_ld64(taddr + lane_base + co, hl);
#pragma unroll
              for (int q4 = 0; q4 < 16; ++q4)
                *reinterpret_cast<float4*>(dl_s + cidx(c, 4 * q4)) =
                    make_float4(hl[4 * q4], hl[4 * q4 + 1], hl[4 * q4 + 2],
                                hl[4 * q4 + 3]);
            }
            named_sync_128();  // the fields are in dl_s
            if (L == 0) stamp(a, Gb, 8);
            ok = __all_sync(0xffffffffu, ok && !*sh.abort);
            if (ok) {
              const bool pvalid = cc < item.nchains;
              const float* jb = jbb + (Gb & 1) * 4096;
              const float* lfb = lf_s + (Gb & 1) * 64 * CC;
              const uint32_t o0 = spins_s[(2 * t) * CC + cc];
              const uint32_t o1 = spins_s[(2 * t + 1) * CC + cc];
              const uint32_t om = hf ? o1 : o0;  // this lane's half
              const float pbeta = beta_s[cc];
              const float scale = ising ? 2.0f : 1.0f;
              const float invbs = invb_s[cc];  // 1 / (pbeta scale), or +inf
              const bool banded = pvalid && invbs < INFINITY;
              const float band0 = banded ? 3e-5f * invbs : 0.0f;
              const float band1 = banded ? 1e-6f * invbs : 0.0f;
              float h[32], w[32];
#pragma unroll
              for (int q4 = 0; q4 < 8; ++q4) {
                const float4 v = *reinterpret_cast<const float4*>(
                    dl_s + cidx(cc, 32 * hf + 4 * q4));
                h[4 * q4 + 0] = v.x;
                h[4 * q4 + 1] = v.y;
                h[4 * q4 + 2] = v.z;
                h[4 * q4 + 3] = v.w;
              }
#pragma unroll
              for (int q4 = 0; q4 < 8; ++q4) {
                const float4 v = *reinterpret_cast<const float4*>(
                    lfb + cidx(cc, 32 * hf + 4 * q4));
                const float av[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                  const int k = 4 * q4 + i;
                  const float tl = av[i] * invbs;  // -|tl|
                  w[k] = ((om >> k) & 1u) ? -tl : tl;
                }
              }
              const uint64_t live64 =
                  kmax >= 64 ? ~0ull : ((1ull << kmax) - 1ull);
              // undecided positions of this lane's half
              uint32_t pend = pvalid ? (uint32_t)(live64 >> (32 * hf)) : 0u;
              uint64_t flips64 = 0ull;
              float dEb = 0.0f;
              const int64_t pchain = item.chain0 + cc;
              if (L == 0) stamp(a, Gb, 9);
    #pragma unroll 1
              for (;;) {
                const uint32_t lo = __reduce_min_sync(
                    0xffffffffu, pend ? (uint32_t)(__ffs(pend) - 1) : 32u);
                // bit k: the sign of h + w at position k.  A position is
                // certainly rejected when h + w and w differ in sign -- the
                // sign of their product, zeros and infinities included, as
                // the one-lane rounds test it -- and w is negative exactly
                // where the spin is 0 (w = -|tl|, tl = a / (beta scale) < 0),
                // so the candidates are (signs ^ spins) & undecided
                uint32_t m[4];
#pragma unroll
                for (int qd = 0; qd < 4; ++qd) {
                  m[qd] = 0u;
                  if (8 * qd + 8 > (int)lo) {
#pragma unroll
                    for (int jj = 7; jj >= 0; --jj) {
                      const int k = 8 * qd + jj;
                      m[qd] = __funnelshift_l(__float_as_uint(h[k] + w[k]),
                                              m[qd], 1);
                    }
                  }
                }
                const uint32_t cand =
                    ((m[0] | (m[1] << 8) | (m[2] << 16) | (m[3] << 24)) ^ om) &
                    pend;
                const uint32_t other = __shfl_xor_sync(0xffffffffu, cand, 16);
                const uint32_t c0 = hf ? other : cand, c1 = hf ? cand : other;
                if (L == 0) count(a, 2, 1);
                if (__all_sync(0xffffffffu, (c0 | c1) == 0u)) break;
                // the chain's next decision (positions up to it decided)
                const int js = c0 ? __ffs(c0) - 1
                                  : (c1 ? 32 + __ffs(c1) - 1 : 0);
                // its field at decision: the lane holding position js has it
                // in registers, corrected by this block's earlier flips in
                // position order (the values and roundings of a rebuild from
                // the loaded fields); a select tree picks it and the partner
                // takes it by shuffle, in every lane so the warp stays
                // converged
                float hsel;
                {
                  const int jl = js & 31;
                  float v16[16], v8[8], v4[4], v2[2];
#pragma unroll
                  for (int i = 0; i < 16; ++i) v16[i] = (jl & 16) ? h[i + 16] : h[i];
#pragma unroll
                  for (int i = 0; i < 8; ++i) v8[i] = (jl & 8) ? v16[i + 8] : v16[i];
#pragma unroll
                  for (int i = 0; i < 4; ++i) v4[i] = (jl & 4) ? v8[i + 4] : v8[i];
#pragma unroll
                  for (int i = 0; i < 2; ++i) v2[i] = (jl & 2) ? v4[i + 2] : v4[i];
                  hsel = (jl & 1) ? v2[1] : v2[0];
                }
                const float hpart = __shfl_xor_sync(0xffffffffu, hsel, 16);
                if ((c0 | c1) == 0u) {
                  pend = 0u;  // the rest rejected: done
                } else {
                  if (c0) {
                    if (hf == 0) pend &= ~((2u << js) - 1u);
                  } else {
                    pend = hf == 0 ? 0u : pend & ~((2u << (js - 32)) - 1u);
                  }
                  const uint64_t bit = 1ull << js;
                  const float hj = (js >> 5) == hf ? hsel : hpart;
                  const bool sbit =
                      ((js < 32 ? o0 >> js : o1 >> (js - 32)) & 1u) != 0u;
                  const float x = sbit ? hj : -hj;
                  const float ak = lfb[cidx(cc, js)];
                  const float th = fminf(
                      fmaf(2.0f * band1, fabsf(ak), fmaf(ak, invbs, 2.0f * band0)),
                      0.0f);
                  bool acc = x >= th;
                  if (!acc) {
                    acc = metropolis_accept_lf(
                        scale * x, pbeta, lf_of(ak),
                        chain_seed(a.seed, a.s.stream_key, pchain),
                        (uint32_t)inst, sweep, (uint32_t)(pchain - chain_base),
                        (uint32_t)(i0 + js));
                  }
                  if (acc) {
                    flips64 |= bit;
                    const float dl = sbit ? -scale : scale;
                    dEb = fmaf(dl, hj, dEb);  // dl h = -dn
                    const float4* row =
                        reinterpret_cast<const float4*>(jb + js * 64 + 32 * hf);
#pragma unroll
                    for (int q4 = 0; q4 < 8; ++q4) {
                      const float4 v = row[q4];
                      h[4 * q4 + 0] = fmaf(dl, v.x, h[4 * q4 + 0]);
                      h[4 * q4 + 1] = fmaf(dl, v.y, h[4 * q4 + 1]);
                      h[4 * q4 + 2] = fmaf(dl, v.z, h[4 * q4 + 2]);
                      h[4 * q4 + 3] = fmaf(dl, v.w, h[4 * q4 + 3]);
                    }
                  }
                }
              }
              if (L == 0) stamp(a, Gb, 10);
              // this lane's half of the chain's A row, once the previous
              // block's MMAs (which read A) are done
              bool a_ok = true;
              if (Gb > G0) a_ok = tc_wait(sh.mma_done, (Gb - 1) & 1, sh, status);
              if (L == 0) stamp(a, Gb, 11);
              const uint32_t fm = (uint32_t)(flips64 >> (32 * hf));
              if (a_ok) {
                unsigned char* rowp = a_row(128 - CC + cc);
#pragma unroll
                for (int kc = 0; kc < C::CPR / 2; ++kc)
                  *reinterpret_cast<uint4*>(rowp +
                                            (C::CPR / 2 * hf + kc) * 128) =
                      make_uint4(0u, 0u, 0u, 0u);
                uint32_t fb = fm;
                while (fb) {
                  const int j = __ffs(fb) - 1;
                  fb &= fb - 1u;
                  a_put(rowp, 32 * hf + j, ((om >> j) & 1u) != 0u);
                }
              }
              if (pvalid) {
                spins_s[(2 * t + hf) * CC + cc] = om ^ fm;
                if (hf == 0) dE_s[cc] += (double)dEb;
              }
              blk_mf = __reduce_max_sync(
                  0xffffffffu, pvalid ? (uint32_t)__popcll(flips64) : 0u);
              if (L == 0) count(a, 0, 1);
              fence_proxy_async();
            }
          } else {
          bool go = q == qt && !*sh.abort;
          // fields of this block: the previous block's critical MMA (not
          // needed for a unit's first block or after a recompute)
          if (go && wait_h && !(RND && F > 1))
            go = tc_wait(sh.h_ready, (Gb - 1) & 1, sh, status);
          if (go) go = tc_wait(&sh.jbb_full[Gb & 1], (Gb >> 1) & 1, sh, status);
          if (go) go = tc_wait(&sh.lf_full[Gb & 1], (Gb >> 1) & 1, sh, status);
          // warp-uniform, so the warp-collective TMEM loads below stay
          // converged
          go = __all_sync(0xffffffffu, go);
          const bool lead = go && c == 0;
          if (lead) stamp(a, Gb, 0);
          // fold 4: block Gb's A buffer is free once the MMAs of block
          // Gb - 2 (its previous user) are done; a unit's first two blocks
          // follow the previous unit's, whose MMAs have all completed
          auto a_buffer_free = [&]() {
            return Gb < G0 + 2 ||
                   tc_wait(&sh.mma_done_b[Gb & 1], ((Gb >> 1) - 1) & 1, sh,
                           status);
          };
          // one sub-block's deltas of chain c into its A row (one copy,
          // seen by every slice's MMA)
          auto put_a = [&](int gg, const float* d) {
            unsigned char* rowp = a_row(
                128 - CC + c + (C::A_NBUF == 2 ? 128 * (int)(Gb & 1) : 0));
            if constexpr (E8) {
              uint32_t pkg[4];
#pragma unroll
              for (int j = 0; j < 16; j += 4)
                pkg[j >> 2] = e4m3_bits(d[j]) | (e4m3_bits(d[j + 1]) << 8) |
                              (e4m3_bits(d[j + 2]) << 16) |
                              (e4m3_bits(d[j + 3]) << 24);
              *reinterpret_cast<uint4*>(rowp + gg * 128) =
                  make_uint4(pkg[0], pkg[1], pkg[2], pkg[3]);
            } else {
              uint32_t pkg[8];
#pragma unroll
              for (int j = 0; j < 16; j += 2)
                pkg[j >> 1] = bf16_bits(d[j]) | (bf16_bits(d[j + 1]) << 16);
              *reinterpret_cast<uint4*>(rowp + (2 * gg) * 128) =
                  make_uint4(pkg[0], pkg[1], pkg[2], pkg[3]);
              *reinterpret_cast<uint4*>(rowp + (2 * gg + 1) * 128) =
                  make_uint4(pkg[4], pkg[5], pkg[6], pkg[7]);
            }
          };
          if (go) {
            tc::fence_after_sync();
            if (lead) stamp(a, Gb, 1);
            const float* jb = jbb + (Gb & 1) * 4096;
            const float* lfb = lf_s + (Gb & 1) * 64 * CC;
            uint32_t o0 = 0u, o1 = 0u;
            if constexpr (RND) {
              // bit k of (o0, o1): spin at position k of the block, made by
              // the helper warps with this block's log-uniforms
              o0 = posb[((Gb & 1) * 2 + 0) * CC + c];
              o1 = posb[((Gb & 1) * 2 + 1) * CC + c];
            } else {
              o0 = spins_s[(2 * t) * CC + c];
              o1 = spins_s[(2 * t + 1) * CC + c];
            }
            uint32_t w0 = o0, w1 = o1;
            float dEb = 0.0f;
            // Decisions in field units: with x = +-h signed so that
            // dn = scale * x, a flip is certain when x >= th and excluded
            // when x < tl.  th and tl bracket log(u) / (beta * scale) by the
            // f32 band of log(u), 3e-5 + 1e-6 |log u| (over three times the
            // error of __logf plus the two roundings of a threshold); in
            // between, the exact f64 rule decides.  With beta <= 0 every
            // flip is accepted (log u < 0 <= beta * dn).
            // Lanes without a chain decide too (their rows of A only touch
            // their own TMEM lanes and their state is never written back):
            // with a zero band (th == tl) they never ask for the exact rule.
            // beta <= 0 makes 1 / beta infinite: th = -inf accepts all.
            const float scale = ising ? 2.0f : 1.0f;
            const float invbs = beta > 0.0f ? 1.0f / (beta * scale) : INFINITY;
            // the band in field units: (3e-5 + 1e-6 |log u|) / (beta scale);
            // none at beta = 0 (t = -inf: every move accepted)
            const bool banded = valid && invbs < INFINITY;
            const float band0 = banded ? 3e-5f * invbs : 0.0f;
            const float band1 = banded ? 1e-6f * invbs : 0.0f;
            // the previous sub-block's deltas (its corrections of this one
            // and its A rows come from registers)
            float dprev[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) dprev[j] = 0.0f;
            bool a_early = false;
            // bit k: position k of the block flipped (chains the CTA holds,
            // positions < kmax)
            uint64_t bflips = 0ull;
            // fields of sub-block g with the corrections of every earlier
            // sub-block of the block
            auto fields = [&](int g, float* hs) {
              if constexpr (!RND) {
                tc::tmem_ld16(taddr + lane_base + co + 16 * g, hs);
              } else if constexpr (F > 1) {
#pragma unroll
                for (int j = 0; j < 16; ++j)
                  hs[j] = 16 * g + j < kmax ? hbuf[(16 * g + j) * CC + c]
                                            : 0.0f;
              } else {
                uint32_t r[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                  const int sp = spos(16 * g + j);
                  r[j] = 0u;
                  if (sp >= 0)
                    r[j] = tc::tmem_ld1_nowait(taddr + lane_base +
                                               (uint32_t)sp);
                }
                tc::tmem_wait_ld16(r);
#pragma unroll
                for (int j = 0; j < 16; ++j) hs[j] = __uint_as_float(r[j]);
              }
              if (lead) stamp(a, Gb, 8 + 3 * g);
              // sub-blocks before the previous one: precomputed by the
              // helpers (fold 2) or from the deltas in shared memory
              if (C::HELP && g >= 2) {
    #pragma unroll
                for (int j = 0; j < 16; ++j)
                  hs[j] += corr_s[((g - 2) * 16 + j) * CC + c];
              } else {
    #pragma unroll 2
                for (int k = 0; k < 16 * (g - 1); ++k) {
                  const float d = dl_s[k * CC + c];
                  const float4* jr =
                      reinterpret_cast<const float4*>(jb + k * 64 + 16 * g);
    #pragma unroll
                  for (int q4 = 0; q4 < 4; ++q4) {
                    const float4 v = jr[q4];
                    hs[4 * q4 + 0] = fmaf(d, v.x, hs[4 * q4 + 0]);
                    hs[4 * q4 + 1] = fmaf(d, v.y, hs[4 * q4 + 1]);
                    hs[4 * q4 + 2] = fmaf(d, v.z, hs[4 * q4 + 2]);
                    hs[4 * q4 + 3] = fmaf(d, v.w, hs[4 * q4 + 3]);
                  }
                }
              }
              // the previous sub-block, from registers
              if (g > 0) {
    #pragma unroll
                for (int kk = 0; kk < 16; ++kk) {
                  const float d = dprev[kk];
                  const float4* jr = reinterpret_cast<const float4*>(
                      jb + (16 * (g - 1) + kk) * 64 + 16 * g);
    #pragma unroll
                  for (int q4 = 0; q4 < 4; ++q4) {
                    const float4 v = jr[q4];
                    hs[4 * q4 + 0] = fmaf(d, v.x, hs[4 * q4 + 0]);
                    hs[4 * q4 + 1] = fmaf(d, v.y, hs[4 * q4 + 1]);
                    hs[4 * q4 + 2] = fmaf(d, v.z, hs[4 * q4 + 2]);
                    hs[4 * q4 + 3] = fmaf(d, v.w, hs[4 * q4 + 3]);
                  }
                }
              }
            };
            // mode-dependent decisions: rounds over the whole block (few
            // flips) or four sequential sub-blocks of 16 spins
            uint64_t flips64 = 0ull;
            if (d64) {
              // ---------------------------------------- block rounds (D64)
              // The block's 64 fields in registers.  A round tests every
              // undecided position against the current fields at once: the
              // first one not certainly rejected (x >= tl) is the next
              // decision -- the positions before it are rejected exactly as
              // the sequential rule rejects them, their fields having seen
              // every earlier flip.  An accepted flip corrects all 64 fields
              // (row js of the diagonal block), and the next round starts
              // after it.  A lane's rounds = its examined candidates + 1;
              // with few flips per block this replaces 64 dependent
              // decisions by a handful of wide ones.
              float h[64];
              if constexpr (!RND) {
                tc::tmem_ld64(taddr + lane_base + co, h);
              } else if constexpr (F > 1) {
#pragma unroll
                for (int k = 0; k < 64; ++k)
                  h[k] = k < kmax ? hbuf[k * CC + c] : 0.0f;
              } else {
                uint32_t r[16];
#pragma unroll
                for (int g = 0; g < 4; ++g) {
#pragma unroll
                  for (int j = 0; j < 16; ++j) {
                    const int sp = spos(16 * g + j);
                    r[j] = 0u;
                    if (sp >= 0)
                      r[j] = tc::tmem_ld1_nowait(taddr + lane_base + (uint32_t)sp);
                  }
                  tc::tmem_wait_ld16(r);
#pragma unroll
                  for (int j = 0; j < 16; ++j) h[16 * g + j] = __uint_as_float(r[j]);
                }
              }
              if (lead) stamp(a, Gb, 8);
              // the block's fields as loaded (a candidate's field at its
              // decision is rebuilt from them, bit for bit), and per position
              // w = sigma |tl|: sign = the spin (+ for s = 1), magnitude the
              // rejection threshold; x >= tl  <=>  (h + w) w >= 0 (exact: a
              // rounded sum or product keeps the sign of the exact one; an
              // underflowing product of opposite signs is -0, still < 0)
#pragma unroll
              for (int q4 = 0; q4 < 16; ++q4)
                *reinterpret_cast<float4*>(dl_s + cidx(c, 4 * q4)) =
                    make_float4(h[4 * q4], h[4 * q4 + 1], h[4 * q4 + 2],
                                h[4 * q4 + 3]);
              float w[64];
#pragma unroll
              for (int k = 0; k < 64; ++k) {
                const float tl = lfb[cidx(c, k)] * invbs;  // -|tl|
                const bool sbit =
                    ((k < 32 ? o0 >> k : o1 >> (k - 32)) & 1u) != 0u;
                w[k] = sbit ? -tl : tl;
              }
              const uint64_t live64 =
                  kmax >= 64 ? ~0ull : ((1ull << kmax) - 1ull);
              uint64_t pend = valid ? live64 : 0ull;  // undecided positions
              if (lead) stamp(a, Gb, 9);
    #pragma unroll 1
              for (;;) {
                // first undecided position over the warp: groups of 8
                // below it are decided in every lane and skipped
                const uint32_t lo = __reduce_min_sync(
                    0xffffffffu,
                    pend ? (uint32_t)(__ffsll((long long)pend) - 1) : 64u);
                // bit k: position k certainly rejected (x < tl)
                uint32_t m[8];
#pragma unroll
                for (int qd = 0; qd < 8; ++qd) {
                  m[qd] = 0u;
                  if (8 * qd + 8 > (int)lo) {
#pragma unroll
                    for (int jj = 7; jj >= 0; --jj) {
                      const int k = 8 * qd + jj;
                      // (h + w) w < 0: the signs differ (a zero sum counts
                      // as rejected: x = tl exactly, safely below the band)
                      const uint32_t x = __float_as_uint((h[k] + w[k]) * w[k]);
                      m[qd] = __funnelshift_l(x, m[qd], 1);
                    }
                  }
                }
                const uint32_t e0 =
                    m[0] | (m[1] << 8) | (m[2] << 16) | (m[3] << 24);
                const uint32_t e1 =
                    m[4] | (m[5] << 8) | (m[6] << 16) | (m[7] << 24);
                const uint64_t cand =
                    ~(((uint64_t)e1 << 32) | (uint64_t)e0) & pend;
                if (lead) count(a, 2, 1);
                if (__all_sync(0xffffffffu, cand == 0ull)) break;
                if (cand == 0ull) pend = 0ull;  // the rest rejected: done
                if (cand != 0ull) {
                  const int js = __ffsll((long long)cand) - 1;
                  const uint64_t bit = 1ull << js;
                  pend &= ~((bit << 1) - 1ull);  // positions <= js decided
                  // the field at decision: loaded value + this block's
                  // earlier flips, in the order the registers took them
                  float hj = dl_s[cidx(c, js)];
                  uint64_t fb = flips64;
                  while (fb) {
                    const int i = __ffsll((long long)fb) - 1;
                    fb &= fb - 1ull;
                    const uint32_t si = (i < 32 ? o0 >> i : o1 >> (i - 32)) & 1u;
                    hj = fmaf(si ? -scale : scale, jb[i * 64 + js], hj);
                  }
                  const bool sbit =
                      ((js < 32 ? o0 >> js : o1 >> (js - 32)) & 1u) != 0u;
                  const float x = sbit ? hj : -hj;
                  const float ak = lfb[cidx(c, js)];
                  const float th = fminf(
                      fmaf(2.0f * band1, fabsf(ak), fmaf(ak, invbs, 2.0f * band0)),
                      0.0f);
                  bool acc = x >= th;
                  if (!acc) {
                    // inside the band: the exact rule
                    acc = metropolis_accept_lf(
                        scale * x, beta, lf_of(ak),
                        chain_seed(a.seed, a.s.stream_key, chain),
                        (uint32_t)inst, sweep, chain_local, (uint32_t)(i0 + js));
                  }
                  if (acc) {
                    flips64 |= bit;
                    const float dl = sbit ? -scale : scale;
                    dEb = fmaf(dl, hj, dEb);  // dl h = -dn
                    const float4* row =
                        reinterpret_cast<const float4*>(jb + js * 64);
#pragma unroll
                    for (int q4 = 0; q4 < 16; ++q4) {
                      const float4 v = row[q4];
                      h[4 * q4 + 0] = fmaf(dl, v.x, h[4 * q4 + 0]);
                      h[4 * q4 + 1] = fmaf(dl, v.y, h[4 * q4 + 1]);
                      h[4 * q4 + 2] = fmaf(dl, v.z, h[4 * q4 + 2]);
                      h[4 * q4 + 3] = fmaf(dl, v.w, h[4 * q4 + 3]);
                    }
                  }
                }
              }
              w0 = o0 ^ (uint32_t)flips64;
              w1 = o1 ^ (uint32_t)(flips64 >> 32);
              if (lead) stamp(a, Gb, 10);

              // A row: zeros, then the flipped positions' deltas, once the
              // MMAs reading this A buffer have completed
              bool a_ok = true;
              if constexpr (C::A_NBUF == 2) {
                a_ok = a_buffer_free();
              } else {
                if (Gb > G0) a_ok = tc_wait(sh.mma_done, (Gb - 1) & 1, sh, status);
              }
              if (lead) stamp(a, Gb, 11);
              if (a_ok) {
                unsigned char* rowp = a_row(
                    128 - CC + c + (C::A_NBUF == 2 ? 128 * (int)(Gb & 1) : 0));
#pragma unroll
                for (int kc = 0; kc < C::CPR; ++kc)
                  *reinterpret_cast<uint4*>(rowp + kc * 128) =
                      make_uint4(0u, 0u, 0u, 0u);
                uint64_t fb = flips64;
                while (fb) {
                  const int j = __ffsll((long long)fb) - 1;
                  fb &= fb - 1ull;
                  const uint32_t sj = (j < 32 ? o0 >> j : o1 >> (j - 32)) & 1u;
                  a_put(rowp, j, sj != 0u);
                }
              }
            } else {
            // four sub-blocks of 16 spins
    #pragma unroll 1
            for (int g = 0; g < 4; ++g) {
              float hs[16];
              fields(g, hs);
              if (lead) stamp(a, Gb, 9 + 3 * g);
              uint32_t wcur = g < 2 ? w0 : w1;
              const int sb = 16 * (g & 1);
              const uint32_t sbits = wcur >> sb;  // spins before the sub-block
              // bit j: position 16 g + j of the block exists (< kmax)
              const int nlive = kmax - 16 * g;
              const uint32_t live_mask =
                  nlive >= 16 ? 0xFFFFu : nlive > 0 ? (1u << nlive) - 1u : 0u;
              float lfv[16];
#pragma unroll
              for (int j = 0; j < 16; ++j) lfv[j] = lfb[cidx(c, 16 * g + j)];

              // fast pass: branch-free decisions on the thresholds; a
              // decision inside the band is only flagged here.  No shared
              // memory stores inside, so the loads of later rows are free to
              // move ahead of earlier decisions
              const uint32_t wsave = wcur;
              const float dEsave = dEb;
              bool unc = false;
              uint32_t flips = 0u;  // bit j: spin 16 g + j flipped
              float dcur[16];
    #pragma unroll
              for (int j = 0; j < 16; ++j) {
                const int k = 16 * g + j;
                const float ak = lfv[j];
                const float tl = ak * invbs;
                const float th =
                    fminf(fmaf(2.0f * band1, fabsf(ak), tl + 2.0f * band0), 0.0f);
                const bool sbit = (sbits >> j) & 1u;
                const float x = sbit ? hs[j] : -hs[j];
                // positions past n have zero fields (x = 0 >= th): their
                // "flips" change no field and no energy and are masked out
                // of the spin word below
                const bool acc = x >= th;
                unc |= !acc && !(x < tl);
                const float dl = acc ? (sbit ? -scale : scale) : 0.0f;
                dcur[j] = dl;
                dEb = fmaf(dl, hs[j], dEb);  // dl h = -dn exactly; 0 if kept
                flips |= acc ? (1u << j) : 0u;
                if (j < 15) {  // exact corrections inside the sub-block
                  const float4* jr =
                      reinterpret_cast<const float4*>(jb + k * 64 + 16 * g);
    #pragma unroll
                  for (int q4 = (j + 1) >> 2; q4 < 4; ++q4) {
                    const float4 v = jr[q4];
                    if (4 * q4 + 0 > j) hs[4 * q4 + 0] = fmaf(dl, v.x, hs[4 * q4 + 0]);
                    if (4 * q4 + 1 > j) hs[4 * q4 + 1] = fmaf(dl, v.y, hs[4 * q4 + 1]);
                    if (4 * q4 + 2 > j) hs[4 * q4 + 2] = fmaf(dl, v.z, hs[4 * q4 + 2]);
                    if (4 * q4 + 3 > j) hs[4 * q4 + 3] = fmaf(dl, v.w, hs[4 * q4 + 3]);
                  }
                }
              }
              wcur ^= (flips & live_mask) << sb;
              if (__any_sync(0xffffffffu, unc)) {
                // rare: the whole sub-block again with the exact f64 rule
                // where needed (out of line)
                RedoCtx rx;
                rx.jb = jb;
                rx.dl_s = dl_s;
                rx.corr_s = corr_s;
                rx.hbuf = hbuf;
                rx.perm_w = perm_s + warp * 64;
                rx.lfb = lfb;
                rx.taddr = taddr + lane_base;
                rx.co = co;
                rx.kmax = kmax;
                rx.c = c;
                rx.g = g;
                rx.i0 = i0;
                rx.sb = sb;
                rx.valid = valid;
                rx.ising = ising;
                rx.beta = beta;
                rx.seed = chain_seed(a.seed, a.s.stream_key, chain);
                rx.inst = (uint32_t)inst;
                rx.sweep = sweep;
                rx.chain_local = chain_local;
                rx.wsave = wsave;
                rx.dEsave = dEsave;
                redo_subblock<F, RND>(rx, &wcur, &dEb);
#pragma unroll
                for (int j = 0; j < 16; ++j) dcur[j] = dl_s[(16 * g + j) * CC + c];
              }
              if (g < 2) w0 = wcur; else w1 = wcur;
              // this sub-block's flips (chains the CTA holds)
              bflips |= (uint64_t)(valid ? ((wcur ^ wsave) >> sb) & 0xFFFFu : 0u)
                        << (16 * g);
#pragma unroll
              for (int j = 0; j < 16; ++j) dl_s[(16 * g + j) * CC + c] = dcur[j];
              // deltas into the A rows.  A is single-buffered: the previous
              // block's MMAs must be done first.  After the second sub-block
              // they usually are (one slice's worth of MMAs); if not (long
              // MMAs at fold 4), the rows wait for the block's end
              if constexpr (C::HELP) {
                // the helpers write the rows of sub-blocks 0 to 2; the last
                // sub-block's here (the previous block's MMAs are long done)
                if (g == 3 && (Gb == G0 || tc_wait(sh.mma_done, (Gb - 1) & 1,
                                                   sh, status)))
                  put_a(3, dcur);
              } else if constexpr (C::APUT) {
                // sub-blocks 0-2 go to the other slices' warps; the last
                // sub-block's rows here, after the previous block's MMAs
                if (g == 2) named_arrive_aput();
                if (g == 3 && a_buffer_free()) put_a(3, dcur);
              } else {
                if (g == 1)
                  a_early =
                      Gb == G0 || mbar_test_wait(sh.mma_done, (Gb - 1) & 1);
                if (a_early && g >= 1) {
                  if (g == 1) put_a(0, dprev);
                  put_a(g, dcur);
                }
              }
#pragma unroll
              for (int j = 0; j < 16; ++j) dprev[j] = dcur[j];
              if (lead) stamp(a, Gb, 10 + 3 * g);
              if (C::HELP && g < 3) named_sync_dec();  // sub-block g published
            }
            if (!C::HELP && !C::APUT && !a_early) {
              if (Gb > G0) {
                if (lead) stamp(a, Gb, 2);
                const bool a_ok =
                    tc_wait(sh.mma_done, (Gb - 1) & 1, sh, status);
                if (lead) stamp(a, Gb, 3);
                if (!a_ok) a_early = true;  // aborting: leave A alone
              }
              if (!a_early) {
    #pragma unroll 1
                for (int gg = 0; gg < 4; ++gg) {
                  float d[16];
#pragma unroll
                  for (int j = 0; j < 16; ++j) d[j] = dl_s[(16 * gg + j) * CC + c];
                  put_a(gg, d);
                }
              }
            }
            flips64 = bflips;
            }  // sequential sub-blocks
            if (valid) {
              if constexpr (!RND) {
                spins_s[(2 * t) * CC + c] = w0;
                spins_s[(2 * t + 1) * CC + c] = w1;
              } else {
                // flips back to the scattered spins
                uint32_t f0 = w0 ^ o0, f1 = w1 ^ o1;
                while (f0) {
                  const int k = __ffs(f0) - 1;
                  f0 &= f0 - 1;
                  const int sp = spos(k);
                  spins_s[(sp >> 5) * CC + c] ^= 1u << (sp & 31);
                }
                while (f1) {
                  const int k = __ffs(f1) - 1;
                  f1 &= f1 - 1;
                  const int sp = spos(32 + k);
                  spins_s[(sp >> 5) * CC + c] ^= 1u << (sp & 31);
                }
              }
              dE_s[c] += (double)dEb;
            }
            blk_mf = __reduce_max_sync(
                0xffffffffu, valid ? (uint32_t)__popcll(flips64) : 0u);
            if (lead) count(a, d64 ? 0 : 1, 1);
            fence_proxy_async();
          } else if (C::APUT && !d64) {
            // one of the three other slices' warps (or every warp after an
            // abort): the A rows of sub-block hr once sub-blocks 0-2 are
            // decided and the previous block's MMAs are done
            named_sync_aput();
            const int hr = (q + 3 - qt) & 3;  // 0, 1, 2 for q = qt+1, +2, +3
            if (hr < 3 && __all_sync(0xffffffffu, !*sh.abort) &&
                a_buffer_free()) {
              float d[16];
#pragma unroll
              for (int j = 0; j < 16; ++j) d[j] = dl_s[(16 * hr + j) * CC + c];
              put_a(hr, d);
            }
            fence_proxy_async();
          } else if (C::HELP && !d64) {
            // helper (the other slice's thread of chain c), or a deciding
            // thread after an abort: same three barriers as the deciding path
            const bool hgo = __all_sync(0xffffffffu, !*sh.abort) && q != qt;
            const float* jb = jbb + (Gb & 1) * 4096;
            float c3[16];
    #pragma unroll
            for (int j = 0; j < 16; ++j) c3[j] = 0.0f;
            named_sync_dec();  // sub-block 0 decided
            bool hok = hgo && valid &&
                       tc_wait(&sh.jbb_full[Gb & 1], (Gb >> 1) & 1, sh, status);
            if (hok) {
              float c2[16];
    #pragma unroll
              for (int j = 0; j < 16; ++j) c2[j] = 0.0f;
    #pragma unroll 2
              for (int k = 0; k < 16; ++k) {
                const float d = dl_s[k * CC + c];
                const float4* jr = reinterpret_cast<const float4*>(jb + k * 64);
    #pragma unroll
                for (int q4 = 0; q4 < 4; ++q4) {
                  const float4 v2 = jr[8 + q4], v3 = jr[12 + q4];
                  c2[4 * q4 + 0] = fmaf(d, v2.x, c2[4 * q4 + 0]);
                  c2[4 * q4 + 1] = fmaf(d, v2.y, c2[4 * q4 + 1]);
                  c2[4 * q4 + 2] = fmaf(d, v2.z, c2[4 * q4 + 2]);
                  c2[4 * q4 + 3] = fmaf(d, v2.w, c2[4 * q4 + 3]);
                  c3[4 * q4 + 0] = fmaf(d, v3.x, c3[4 * q4 + 0]);
                  c3[4 * q4 + 1] = fmaf(d, v3.y, c3[4 * q4 + 1]);
                  c3[4 * q4 + 2] = fmaf(d, v3.z, c3[4 * q4 + 2]);
                  c3[4 * q4 + 3] = fmaf(d, v3.w, c3[4 * q4 + 3]);
                }
              }
    #pragma unroll
              for (int j = 0; j < 16; ++j) corr_s[j * CC + c] = c2[j];
            }
            // A rows of the decided sub-blocks below `upto`, once the
            // previous block's MMAs are done with A (tested without waiting
            // until the last call, so the deciders never wait for it here)
            int na = 0;
            auto put_decided = [&](int upto, bool block) {
              if (!hgo || na >= upto) return;
              bool ready =
                  Gb == G0 || mbar_test_wait(sh.mma_done, (Gb - 1) & 1);
              if (!ready && block)
                ready = tc_wait(sh.mma_done, (Gb - 1) & 1, sh, status);
              if (!ready) return;
              for (; na < upto; ++na) {
                float d[16];
#pragma unroll
                for (int j = 0; j < 16; ++j)
                  d[j] = dl_s[(16 * na + j) * CC + c];
                put_a(na, d);
              }
            };
            put_decided(1, false);
            named_sync_dec();  // sub-block 1 decided; corrections of 2 out
            if (hok) {
    #pragma unroll 2
              for (int k = 16; k < 32; ++k) {
                const float d = dl_s[k * CC + c];
                const float4* jr = reinterpret_cast<const float4*>(jb + k * 64);
    #pragma unroll
                for (int q4 = 0; q4 < 4; ++q4) {
                  const float4 v3 = jr[12 + q4];
                  c3[4 * q4 + 0] = fmaf(d, v3.x, c3[4 * q4 + 0]);
                  c3[4 * q4 + 1] = fmaf(d, v3.y, c3[4 * q4 + 1]);
                  c3[4 * q4 + 2] = fmaf(d, v3.z, c3[4 * q4 + 2]);
                  c3[4 * q4 + 3] = fmaf(d, v3.w, c3[4 * q4 + 3]);
                }
              }
    #pragma unroll
              for (int j = 0; j < 16; ++j) corr_s[(16 + j) * CC + c] = c3[j];
            }
            put_decided(2, false);
            named_sync_dec();  // sub-block 2 decided; corrections of 3 out
            put_decided(3, true);
            fence_proxy_async();
          }
          }
          if (lane == 0) stat_s[(Gb & 1) * 4 + warp] = blk_mf;
          named_sync_128();
          {
            uint32_t mf = 0u;
#pragma unroll
            for (int w4 = 0; w4 < 4; ++w4) mf = max(mf, stat_s[(Gb & 1) * 4 + w4]);
            d64 = a.decision_mode == 1 ||
                  (a.decision_mode == 0 && (int)mf <= a.round_limit);
          }
          if (threadIdx.x == 0) {
            stamp(a, Gb, 4);
            mbar_arrive(sh.a_full);
            mbar_arrive(&sh.jbb_free[Gb & 1]);
            mbar_arrive(&sh.lf_free[Gb & 1]);
          }
        }  // blocks

        // ------------------------------------------------ end of the sweep
        // energy of the sweep's last state, per-chain best (strict <,
        // pysa/simulation.py:150-171), then the exchange of the item's reads
        if (q == 0 && valid && !*sh.abort) {
          const float e_f = (float)(e0_s[c] + dE_s[c]);
          if (e_f < __ldcg(a.s.best_energy + chain)) {
            a.s.best_energy[chain] = e_f;
            a.s.best_sweep[chain] = (int32_t)sweep;
            for (int w = 0; w < words; ++w)
              a.s.best_spins[chain * a.p.words + w] = spins_s[w * CC + c];
          }
          e0_s[c] = (double)e_f;
          dE_s[c] = 0.0;
          ex_E[c] = e_f;
        }
        named_sync_128();
        if (a.fuse_exchange && a.use_pt &&
            exchange_after(a.exchange_every, sweep) && !*sh.abort) {
          // pysa/utils.py:44-58 per read, warp per read: pairs (R-1, R-2),
          // (R-2, R-3), ... in order; uniforms of stream (PT, inst, sweep,
          // read, pair)
          const int R = a.p.replicas[inst];
          const float* betas = a.p.ladder + a.p.ladder_off[inst];
          const int nreads = item.nchains / R;
          int32_t* B = ex_B + warp * CC;
          uint32_t* X = ex_X + warp * CC;
          float* Lx = ex_L + warp * CC;
          float* Bt = ex_T + warp * CC;
          for (int k = lane; k < R; k += 32) Bt[k] = betas[k];
          for (int r = warp; r < nreads; r += 4) {
            const int64_t gbase = item.chain0 + (int64_t)r * R;
            const uint32_t lread = (uint32_t)((gbase - chain_base) / R);
            const float* E = ex_E + r * R;
            for (int k = lane; k < R; k += 32) {
              B[k] = __ldcg(a.s.beta_idx + gbase + k);
              if (k < R - 1) {
                const uint32_t x = draw1(a.seed, TAG_PT, (uint32_t)inst, sweep,
                                         lread, (uint32_t)k);
                X[k] = x;
                Lx[k] = log_uniform_f32(x);
              }
            }
            __syncwarp();
            // The pass over pairs (R-1, R-2), (R-2, R-3), ... is serial, but
            // only the replica entering slot k1 carries from pair to pair:
            // slot k2 is untouched until pair k.  So every pair's other
            // replica, its energy and the betas' difference are read by the
            // lanes up front, and the pass keeps the carried replica and
            // its energy in registers (same arithmetic, same decisions).
            int32_t* B2 = ex_B2 + warp * CC;
            float* E2 = ex_E2 + warp * CC;
            float* Dk = ex_D + warp * CC;
            for (int k = lane; k < R - 1; k += 32) {
              const int k1 = R - k - 1, k2 = R - k - 2;
              const int b2 = B[k2];
              B2[k] = b2;
              E2[k] = E[b2];
              Dk[k] = __fsub_rn(Bt[k1], Bt[k2]);
            }
            __syncwarp();
            if (lane == 0 && R > 1) {
              int cb = B[R - 1];
              float ce = E[cb];
              for (int k = 0; k < R - 1; ++k) {
                const int b2 = B2[k];
                const float e2 = E2[k];
                const float de = __fmul_rn(__fsub_rn(ce, e2), Dk[k]);
                const bool sw = pt_accept_lf(de, Lx[k], X[k]);
                B[R - k - 1] = sw ? b2 : cb;   // final: no later pair
                cb = sw ? cb : b2;
                ce = sw ? ce : e2;
              }
              B[0] = cb;
            }
            __syncwarp();
            for (int k = lane; k < R; k += 32) {
              a.s.beta_idx[gbase + k] = B[k];
              a.s.chain_beta[gbase + B[k]] = Bt[k];
              beta_s[r * R + B[k]] = Bt[k];
              invb_s[r * R + B[k]] = inv_bs(Bt[k]);
            }
            __syncwarp();
          }
        }
        named_sync_128();
      }  // sweeps

      // ----------------------------------------------------------- epilogue
      if (!*sh.abort) mmas_done_through<C::A_NBUF>(Gend - 1, sh, status);
      tc::fence_after_sync();
      if (threadIdx.x == 0) stamp_cta(a, 2);
      if (__all_sync(0xffffffffu, !*sh.abort)) {
        for (int j0 = 0; j0 < S; j0 += 32) {
          float v[32];
          tc::tmem_ld32(taddr + lane_base + j0, v);
#pragma unroll
          for (int i = 0; i < 32; ++i) stg[lane * 33 + i] = v[i];
          __syncwarp();
          const int col = w_q * S + j0 + 4 * (lane & 7);
#pragma unroll
          for (int it = 0; it < 8; ++it) {
            const int rr = 4 * it + (lane >> 3);
            const int cr = w_c0 + rr;
            if (cr < item.nchains && col < n) {
              const float* sv = stg + rr * 33 + 4 * (lane & 7);
              float* f =
                  a.fields + (item.chain0 + cr) * (int64_t)a.field_ld + col;
              if (col + 4 <= n) {
                *reinterpret_cast<float4*>(f) =
                    make_float4(sv[0], sv[1], sv[2], sv[3]);
              } else {
                f[0] = sv[0];
                if (col + 1 < n) f[1] = sv[1];
                if (col + 2 < n) f[2] = sv[2];
              }
            }
          }
          __syncwarp();
        }
      }
      tc::fence_before_sync();
      named_sync_128();
      if (threadIdx.x == 0) stamp_cta(a, 3);
      if (q == 0 && valid && !*sh.abort) {
        a.s.energies[chain] = (float)e0_s[c];
        for (int w = 0; w < words; ++w)
          a.s.spins[chain * a.p.words + w] = spins_s[w * CC + c];
      }
    } else if (warp == 4) {
      // ============================================================== MMA
      if (lane == 0) {
        // rows [r_lo, r_hi) of the kTW-row B tile in `slot` against A slice
        // qq, into the field columns kTW j + r_lo ...
        // Descriptors of the A region's and the B ring's starts, built once:
        // a view or stage further in adds its byte offset / 16 to the
        // address field (shared addresses stay below 2^18, so it never
        // carries out).  The MMA thread shares its sub-partition with a
        // deciding warp that is nearly always ready, and every instruction
        // on its path waits for an issue slot, so it keeps few instructions
        // per MMA (microbenchmark: a block's MMA sequence beside such a warp
        // 10.3k cycles with descriptors built per call, 4.9k prebuilt).
        const uint64_t a_desc0 =
            tc::smem_desc(smem_base + (uint32_t)C::A_OFF, 128, C::SBO);
        const uint64_t b_desc0 =
            tc::smem_desc(smem_base + (uint32_t)C::B_OFF, 128, C::SBO);
        auto mma_rows = [&](uint32_t slot, int qq, int j, int r_lo, int r_hi,
                            uint32_t acc, int ab) {
          if (r_hi <= r_lo) return;
          const uint32_t idesc =
              r_hi - r_lo == kTW
                  ? idesc_full
                  : (E8 ? tc::idesc_e4m3(128, r_hi - r_lo)
                        : tc::idesc_bf16(128, r_hi - r_lo));
          // slice qq's view: 128 rows starting (128 - CC - qq CC) rows in;
          // K steps (16 BF16 or 32 E4M3 elements: two core matrices) are
          // 256 bytes apart: 16 in the address field
          const uint64_t ad =
              a_desc0 +
              (uint64_t)((uint32_t)((128 - CC - qq * CC + 128 * ab) >> 3) *
                         (C::SBO >> 4));
          const uint64_t bd =
              b_desc0 + (uint64_t)(slot * (uint32_t)(C::B_STAGE >> 4) +
                                   (uint32_t)(r_lo / 8) * (C::SBO >> 4));
          if constexpr (E8) {
#pragma unroll
            for (int ks = 0; ks < 2; ++ks)
              tc::mma_e4m3(taddr + kTW * j + r_lo, ad + 16u * ks,
                           bd + 16u * ks, idesc, (acc | (uint32_t)ks) ? 1u : 0u);
          } else {
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
              tc::mma_bf16(taddr + kTW * j + r_lo, ad + 16u * ks,
                           bd + 16u * ks, idesc, (acc | (uint32_t)ks) ? 1u : 0u);
          }
        };
        bool ok = true;
        for (int s = 0; s < KU && ok; ++s) {
          if (rc_at(s)) {
            for (int t = 0; t < NB && ok; ++t) {
              if (!tc_wait(sh.rc_full, RG & 1, sh, status)) {
                ok = false;
                break;
              }
              tc::fence_after_sync();
              for (int j = 0; j < NT && ok; ++j) {
                const int width = S - kTW * j < kTW ? S - kTW * j : kTW;
                for (int term = 0; term < T && ok; ++term) {
                  for (int qq = 0; qq < F; ++qq) {
                    const uint32_t slot = u % C::NS;
                    if (!tc_wait(&sh.full[slot], (u / C::NS) & 1, sh, status)) {
                      ok = false;
                      break;
                    }
                    tc::fence_after_sync();
                    mma_rows(slot, qq, j, 0, width,
                             (t | term | qq) ? 1u : 0u, 0);
                    tc::commit(&sh.free_[slot]);
                    ++u;
                  }
                }
              }
              if (!ok) break;
              tc::commit(sh.rc_done);
              ++RG;
            }
          }
          for (int t = 0; t < NB && ok; ++t) {
            const uint32_t Gb = G0 + (uint32_t)(s * NB + t);
            // the next block's 64 columns (next sweep's first block after the
            // last): slice qn, tile jf, rows r0 .. r0+63.  Worked out before
            // the wait: the deciders wait for the MMAs that use them
            const bool has_next = Gb + 1 < Gend;
            const int tn = t + 1 < NB ? t + 1 : 0;
            const int qn = (64 * tn) / S, cn = 64 * tn - qn * S;
            const int jf = has_next ? cn / kTW : 0, r0 = cn % kTW;
            asm volatile("" ::"r"(jf), "r"(r0), "r"(qn));
            if (!tc_wait(sh.a_full, Gb & 1, sh, status)) {
              ok = false;
              break;
            }
            stamp(a, Gb, 5);
            tc::fence_after_sync();
            const int ab = C::A_NBUF == 2 ? (int)(Gb & 1) : 0;
            // stage order: slices from qn on, tiles inside (the critical
            // one first), terms innermost -- consecutive stages write
            // different accumulator tiles, so their MMAs need not wait for
            // one another (the producer issues the same order)
            for (int k = 0; k < F && ok; ++k) {
              const int qq = (qn + k) % F;
              for (int jj = 0; jj < NT && ok; ++jj) {
                const int j = jj == 0 ? jf : (jj <= jf ? jj - 1 : jj);
                const int width = S - kTW * j < kTW ? S - kTW * j : kTW;
                // random order: the next block's columns are scattered, so
                // no tile is critical; h_ready follows the whole block
                const bool crit = !RND && jj == 0 && k == 0 && has_next;
                for (int term = 0; term < T; ++term) {
                  const uint32_t slot = (u + term) % C::NS;
                  if (k * NT + jj < 4 && term == 0) stamp(a, Gb, 20 + k * NT + jj);
                  if (!tc_wait(&sh.full[slot], ((u + term) / C::NS) & 1, sh,
                               status)) {
                    ok = false;
                    break;
                  }
                  if (k * NT + jj < 4 && term == 0) stamp(a, Gb, 12 + k * NT + jj);
                  tc::fence_after_sync();
                  if (crit)
                    mma_rows(slot, qq, j, r0, r0 + 64, 1u, ab);
                  else
                    mma_rows(slot, qq, j, 0, width, 1u, ab);
                }
                if (!ok) break;
                if (crit) {
                  // the next block's decisions may start once these land
                  tc::commit(sh.h_ready);
                  stamp(a, Gb, 6);
                  for (int term = 0; term < T; ++term) {
                    const uint32_t slot = (u + term) % C::NS;
                    mma_rows(slot, qq, j, 0, r0, 1u, ab);
                    mma_rows(slot, qq, j, r0 + 64, width, 1u, ab);
                  }
                }
                for (int term = 0; term < T; ++term)
                  tc::commit(&sh.free_[(u + term) % C::NS]);
                u += T;
              }
            }
            if (!ok) break;
            if (!has_next || RND) {
              tc::commit(sh.h_ready);  // one phase per block
              if (RND) stamp(a, Gb, 6);
            }
            tc::commit(sh.mma_done);
            if (C::A_NBUF == 2) tc::commit(&sh.mma_done_b[Gb & 1]);
          }
        }
        if (!ok) *sh.abort = 1;
      }
    } else if (warp == 5) {
      // ========================================================= producer
      if (lane == 0) {
        const uint16_t* Bp = a.tc_b + item.b_off;
        const float* D = a.tc_diag + item.diag_off;
        const size_t tile_bytes = (size_t)kTW * C::ROW_B;
        // diagonal block of global block Gx (block (Gx - G0) % NB of the
        // unit) into buffer Gx & 1, once block Gx - 2 has released it
        // random order: the sweep's repacked slot (same offsets)
        auto rand_slot = [&](int s_) {
          return (int64_t)((sweep_first + (uint32_t)s_) %
                           (uint32_t)(a.rand_slots > 0 ? a.rand_slots : 1));
        };
        auto issue_jbb = [&](uint32_t Gx) {
          if (Gx >= 2 &&
              !tc_wait(&sh.jbb_free[Gx & 1], ((Gx >> 1) - 1) & 1, sh, status))
            return false;
          const int tx = (int)((Gx - G0) % (uint32_t)NB);
          const float* Dx = D;
          if (RND)
            Dx = a.rand_diag + rand_slot((int)((Gx - G0) / (uint32_t)NB)) *
                                   a.rand_diag_stride + item.diag_off;
          uint64_t* bar = &sh.jbb_full[Gx & 1];
          mbar_expect_tx_arrive(bar, 16384);
          bulk_g2s(smem + C::JBB_OFF + (Gx & 1) * 16384, Dx + (size_t)tx * 4096,
                   16384, bar);
          return true;
        };
        auto issue_stage = [&](const uint16_t* Bsrc, int t, int term, int qq,
                               int j) {
          const uint32_t slot = u % C::NS;
          if (u >= (uint32_t)C::NS &&
              !tc_wait(&sh.free_[slot], ((u / C::NS) - 1) & 1, sh, status))
            return false;
          const int width = S - kTW * j < kTW ? S - kTW * j : kTW;
          const size_t src =
              ((((size_t)t * T + term) * F + qq) * NT + j) * tile_bytes;
          const uint32_t bytes = (uint32_t)width * C::ROW_B;
          mbar_expect_tx_arrive(&sh.full[slot], bytes);
          bulk_g2s(smem + C::B_OFF + slot * C::B_STAGE,
                   reinterpret_cast<const unsigned char*>(Bsrc) + src, bytes,
                   &sh.full[slot]);
          ++u;
          return true;
        };
        auto issue_jbb_t = [&](uint32_t Gx) {
          const bool r = issue_jbb(Gx);
          if (r) jbb_last = Gx;
          return r;
        };
        bool ok = issue_jbb_t(G0);
        for (int s = 0; s < KU && ok; ++s) {
          if (rc_at(s)) {
            for (int t = 0; t < NB && ok; ++t)
              for (int j = 0; j < NT && ok; ++j)
                for (int term = 0; term < T && ok; ++term)
                  for (int qq = 0; qq < F && ok; ++qq)
                    ok = issue_stage(Bp, t, term, qq, j);
          }
          const uint16_t* Bs =
              RND ? a.rand_b + rand_slot(s) * a.rand_b_stride + item.b_off
                  : Bp;
          for (int t = 0; t < NB && ok; ++t) {
            const uint32_t Gb = G0 + (uint32_t)(s * NB + t);
            // the next block's diagonal block lands while this one is decided
            if (Gb + 1 < Gend) ok = issue_jbb_t(Gb + 1);
            const bool has_next = Gb + 1 < Gend;
            const int tn = (t + 1) % NB;
            const int jf = has_next ? ((64 * tn) % S) / kTW : 0;
            const int qn = (64 * tn) / S;
            for (int k = 0; k < F && ok; ++k)
              for (int jj = 0; jj < NT && ok; ++jj) {
                const int j = jj == 0 ? jf : (jj <= jf ? jj - 1 : jj);
                for (int term = 0; term < T && ok; ++term) {
                  ok = issue_stage(Bs, t, term, (qn + k) % F, j);
                  if (k * NT + jj < 4 && term == 0) stamp(a, Gb, 16 + k * NT + jj);
                }
              }
            stamp(a, Gb, 7);
          }
        }
        if (!ok) *sh.abort = 1;
      }
    } else {
      // ================================= log-uniforms of the next blocks
      const int hid = threadIdx.x - 192;
      for (int s = 0; s < KU; ++s) {
        const uint32_t sweep = sweep_first + (uint32_t)s;
        for (int t = 0; t < NB; ++t) {
          const uint32_t Gb = G0 + (uint32_t)(s * NB + t);
          bool go = !*sh.abort;
          if (go && Gb >= 2)
            go = tc_wait(&sh.lf_free[Gb & 1], ((Gb >> 1) - 1) & 1, sh, status);
          if (go) {
            float* out = lf_s + (Gb & 1) * 64 * CC;
            for (int it = hid; it < CC * 16; it += 64) {
              const int c2 = it % CC, quad = it / CC;
              const uint32_t cl = (uint32_t)(item.chain0 + c2 - chain_base);
              const uint64_t sk =
                  c2 < item.nchains
                      ? chain_seed(a.seed, a.s.stream_key, item.chain0 + c2)
                      : a.seed;
              uint32_t x[4];
              draw4(sk, TAG_SWEEP, (uint32_t)inst, sweep, cl,
                    (uint32_t)(16 * t + quad), x);
              // a = log u - m: the rejection bound in the log domain, m =
              // 3e-5 + 1e-6 |log u| the band of the f32 log (over three
              // times the error of __logf plus the roundings of a
              // threshold); the deciders scale it by 1 / (beta scale)
              float4 v;
              v.x = log_uniform_f32(x[0]);
              v.y = log_uniform_f32(x[1]);
              v.z = log_uniform_f32(x[2]);
              v.w = log_uniform_f32(x[3]);
              v.x -= fmaf(1e-6f, fabsf(v.x), 3e-5f);
              v.y -= fmaf(1e-6f, fabsf(v.y), 3e-5f);
              v.z -= fmaf(1e-6f, fabsf(v.z), 3e-5f);
              v.w -= fmaf(1e-6f, fabsf(v.w), 3e-5f);
              *reinterpret_cast<float4*>(out + cidx(c2, 4 * quad)) = v;
            }
          }
          if constexpr (RND) {
            // spin words of this block in position order.  Its spins are
            // not touched by earlier blocks of the same sweep; the previous
            // sweep's last block must have finished (blocks Gb-2 and older
            // have, by the lf_free wait above)
            const uint32_t Gs = G0 + (uint32_t)(s * NB);
            if (go && Gs > G0 && Gb - Gs <= 1)
              go = tc_wait(&sh.lf_free[(Gs - 1) & 1], ((Gs - 1) >> 1) & 1, sh,
                           status);
            if (go) {
              const int32_t* pr =
                  a.perm + ((int64_t)(sweep % (uint32_t)a.perm_slots) *
                                a.p.num_instances + inst) * a.p.max_n +
                  64 * t;
              const int kmax = n - 64 * t < 64 ? n - 64 * t : 64;
              for (int c2 = hid; c2 < CC; c2 += 64) {
                uint32_t w0 = 0u, w1 = 0u;
                for (int k = 0; k < kmax; ++k) {
                  const int sp = pr[k];
                  const uint32_t bit =
                      (spins_s[(sp >> 5) * CC + c2] >> (sp & 31)) & 1u;
                  if (k < 32) w0 |= bit << k; else w1 |= bit << (k - 32);
                }
                posb[((Gb & 1) * 2 + 0) * CC + c2] = w0;
                posb[((Gb & 1) * 2 + 1) * CC + c2] = w1;
              }
            }
          }
          named_sync_helpers();
          if (hid == 0) mbar_arrive(&sh.lf_full[Gb & 1]);
        }
      }
    }

    // ------------------------------------------------------- unit end
    __threadfence();  // this unit's global stores before its done flag
    G = Gend;
    RG = RG0 + (uint32_t)(n_rc * NB);
    __syncwarp();  // single-lane roles (MMA, producer) rejoin their warps
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (*sh.abort) {
      // Aborted (a bounded wait ran out): every role has stopped issuing.
      // Asynchronous work already in flight lands before the CTA frees its
      // tensor memory and exits (the next unit-queue step ends it): the
      // MMAs issued so far, and the producer's last NS ring stages and last
      // two diagonal blocks (older copies were waited for before their
      // buffers were reused).
      if (warp == 4 && lane == 0) {
        tc::commit(sh.drain);
        drain_wait(sh.drain, 0);
      }
      if (warp == 5 && lane == 0) {
        const uint32_t lo =
            u - u_first > (uint32_t)C::NS ? u - (uint32_t)C::NS : u_first;
        for (uint32_t x = lo; x < u; ++x)
          drain_wait(&sh.full[x % C::NS], (x / C::NS) & 1);
        if (jbb_last != 0xFFFFFFFFu) {
          drain_wait(&sh.jbb_full[jbb_last & 1], (jbb_last >> 1) & 1);
          if (jbb_last > G0)
            drain_wait(&sh.jbb_full[(jbb_last - 1) & 1],
                       ((jbb_last - 1) >> 1) & 1);
        }
      }
      __syncwarp();
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
    }
    if (threadIdx.x == 0) {
      stamp_cta(a, 4);
      __threadfence();  // this unit's stores before its done flag
      atomicExch(reinterpret_cast<int*>(a.sched + 2 + un_item),
                 un_first + KU);
    }
  }

  // ------------------------------------------------------------ teardown
  if (threadIdx.x == 0) {
    __threadfence();
    const uint32_t fin = atomicAdd(reinterpret_cast<unsigned*>(a.sched + 1), 1u);
    if (fin == gridDim.x - 1 && a.advance_counter)
      *a.s.sweep_counter += (int64_t)a.unit_sweeps * a.units_per_item;
  }
  __syncwarp();
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(taddr, kCols);
  }
}

#ifndef PYSA_GB_TC_E8_UNIT
// -------------------------------------------------------------- packing
// B tiles: for block t, term, slice qq, tile j: rows r < width (column
// qq*S + kTW j + r), k < 64 (spin 64 t + k), canonical no-swizzle K-major
// order: ((r / 8) * 8 + k / 8) * 64 + (r % 8) * 8 + k % 8 (bf16 elements).
__global__ void k_pack_tc_b(const float* Jt, int ld, int n, int F, int terms,
                            uint16_t* out) {
  const int NP = (n + 64 * F - 1) / (64 * F) * (64 * F);
  const int S = NP / F, NB = (n + 63) / 64, NT = (S + kTW - 1) / kTW;
  const int64_t tile = (int64_t)kTW * 64;
  const int64_t total = (int64_t)NB * terms * F * NT * tile;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t rest = e;
    const int within = (int)(rest % tile);
    rest /= tile;
    const int j = (int)(rest % NT);
    rest /= NT;
    const int qq = (int)(rest % F);
    rest /= F;
    const int term = (int)(rest % terms);
    const int t = (int)(rest / terms);
    const int cm = within / 64, inside = within % 64;
    const int r = (cm / 8) * 8 + inside / 8;
    const int k = (cm % 8) * 8 + inside % 8;
    const int row = 64 * t + k, col = qq * S + kTW * j + r;
    float v = 0.0f;
    if (row < n && col < n && r < kTW && kTW * j + r < S)
      v = Jt[(int64_t)row * ld + col];
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
    const __nv_bfloat16 o = term == 0 ? hi : lo;
    out[e] = *reinterpret_cast<const uint16_t*>(&o);
  }
}

// E4M3 tiles (one term, couplings exact in E4M3): the same tiles with
// 16-byte core-matrix rows of 16 elements, ((r / 8) * 4 + k / 16) * 128 +
// (r % 8) * 16 + k % 16 (bytes).
__global__ void k_pack_tc_b8(const float* Jt, int ld, int n, int F,
                             unsigned char* out) {
  const int NP = (n + 64 * F - 1) / (64 * F) * (64 * F);
  const int S = NP / F, NB = (n + 63) / 64, NT = (S + kTW - 1) / kTW;
  const int64_t tile = (int64_t)kTW * 64;
  const int64_t total = (int64_t)NB * F * NT * tile;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t rest = e;
    const int within = (int)(rest % tile);
    rest /= tile;
    const int j = (int)(rest % NT);
    rest /= NT;
    const int qq = (int)(rest % F);
    const int t = (int)(rest / F);
    const int cm = within / 128, inside = within % 128;
    const int r = (cm / 4) * 8 + inside / 16;
    const int k = (cm % 4) * 16 + inside % 16;
    const int row = 64 * t + k, col = qq * S + kTW * j + r;
    float v = 0.0f;
    if (row < n && col < n && r < kTW && kTW * j + r < S)
      v = Jt[(int64_t)row * ld + col];
    out[e] = (unsigned char)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
  }
}

// Diagonal blocks: out[t][k][k2] = J^T[64t + k][64t + k2] (f32).
__global__ void k_pack_tc_diag(const float* Jt, int ld, int n, float* out) {
  const int NB = (n + 63) / 64;
  const int64_t total = (int64_t)NB * 4096;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(e / 4096), k = (int)(e % 4096) / 64, k2 = (int)(e % 64);
    const int row = 64 * t + k, col = 64 * t + k2;
    out[e] = (row < n && col < n) ? Jt[(int64_t)row * ld + col] : 0.0f;
  }
}

// Random order: the same tiles and diagonal blocks with spin position
// 64 t + k standing for spin perm[64 t + k] (rows of J^T gathered; field
// columns stay natural in the tiles, both sides permuted in the diagonal
// blocks).  Grid: x over elements, y = instance, z = sweep ahead.
__global__ void k_repack_tc(const pysa_gb_problems p, int terms,
                            const int64_t* inst_off, const int32_t* perm,
                            int perm_slots, const int64_t* sweep_counter,
                            int slots, uint16_t* b_out, int64_t b_stride,
                            float* diag_out, int64_t diag_stride) {
  const int inst = blockIdx.y;
  const int64_t boff = inst_off[2 * inst], doff = inst_off[2 * inst + 1];
  if (boff < 0) return;
  const int n = p.n[inst], ld = p.ld[inst];
  const float* Jt = p.J + p.j_off[inst];
  const uint32_t sweep = (uint32_t)(*sweep_counter) + blockIdx.z;
  const int32_t* pi =
      perm + ((int64_t)(sweep % (uint32_t)perm_slots) * p.num_instances +
              inst) * p.max_n;
  const int64_t slot = sweep % (uint32_t)slots;
  const int F = n <= 512 ? 1 : (n <= 1024 ? 2 : 4);
  const int NP = (n + 64 * F - 1) / (64 * F) * (64 * F);
  const int S = NP / F, NB = (n + 63) / 64, NT = (S + kTW - 1) / kTW;
  const int64_t tile = (int64_t)kTW * 64;
  const int64_t tb = (int64_t)NB * terms * F * NT * tile;
  const int64_t td = (int64_t)NB * 4096;
  uint16_t* bo = b_out + slot * b_stride + boff;
  float* dout = diag_out + slot * diag_stride + doff;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tb + td;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (e < tb) {
      int64_t rest = e;
      const int within = (int)(rest % tile);
      rest /= tile;
      const int j = (int)(rest % NT);
      rest /= NT;
      const int qq = (int)(rest % F);
      rest /= F;
      const int term = (int)(rest % terms);
      const int t = (int)(rest / terms);
      const int cm = within / 64, inside = within % 64;
      const int r = (cm / 8) * 8 + inside / 8;
      const int k = (cm % 8) * 8 + inside % 8;
      const int pos = 64 * t + k, col = qq * S + kTW * j + r;
      float v = 0.0f;
      if (pos < n && col < n && kTW * j + r < S)
        v = Jt[(int64_t)pi[pos] * ld + col];
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
      const __nv_bfloat16 o = term == 0 ? hi : lo;
      bo[e] = *reinterpret_cast<const uint16_t*>(&o);
    } else {
      const int64_t d = e - tb;
      const int t = (int)(d / 4096), k = (int)(d % 4096) / 64,
                k2 = (int)(d % 64);
      const int a1 = 64 * t + k, a2 = 64 * t + k2;
      dout[d] = (a1 < n && a2 < n) ? Jt[(int64_t)pi[a1] * ld + pi[a2]] : 0.0f;
    }
  }
}

cudaError_t launch_repack_tc(const pysa_gb_problems& p, int terms,
                             const int64_t* inst_off, const int32_t* perm,
                             int perm_slots, const int64_t* sweep_counter,
                             int count, int slots, uint16_t* b_out,
                             int64_t b_stride, float* diag_out,
                             int64_t diag_stride, cudaStream_t st) {
  if (count <= 0 || p.num_instances <= 0) return cudaSuccess;
  const int64_t per = tc_b_elems(p.max_n, terms) + tc_diag_elems(p.max_n);
  int bx = (int)((per + 255) / 256);
  if (bx > 1024) bx = 1024;
  dim3 grid((unsigned)bx, (unsigned)p.num_instances, (unsigned)count);
  k_repack_tc<<<grid, 256, 0, st>>>(p, terms, inst_off, perm, perm_slots,
                                    sweep_counter, slots, b_out, b_stride,
                                    diag_out, diag_stride);
  return cudaGetLastError();
}

int tc_fold_for(int n) {
  if (n <= 512) return 1;
  if (n <= 1024) return 2;
  if (n <= 2048) return 4;
  return -1;
}

int64_t tc_b_elems(int n, int terms) {
  const int F = tc_fold_for(n);
  const int NP = (n + 64 * F - 1) / (64 * F) * (64 * F);
  const int S = NP / F, NB = (n + 63) / 64, NT = (S + kTW - 1) / kTW;
  return (int64_t)NB * terms * F * NT * kTW * 64;
}

int64_t tc_diag_elems(int n) { return (int64_t)((n + 63) / 64) * 4096; }

cudaError_t launch_pack_tc(const float* Jt, int ld, int n, int terms,
                           bool e8, uint16_t* b_out, float* diag_out,
                           cudaStream_t st) {
  const int F = tc_fold_for(n);
  int64_t tb = tc_b_elems(n, terms);
  int blocks = (int)((tb + 255) / 256);
  if (blocks > 8192) blocks = 8192;
  if (e8)
    k_pack_tc_b8<<<blocks, 256, 0, st>>>(
        Jt, ld, n, F, reinterpret_cast<unsigned char*>(b_out));
  else
    k_pack_tc_b<<<blocks, 256, 0, st>>>(Jt, ld, n, F, terms, b_out);
  int64_t td = tc_diag_elems(n);
  blocks = (int)((td + 255) / 256);
  if (blocks > 8192) blocks = 8192;
  k_pack_tc_diag<<<blocks, 256, 0, st>>>(Jt, ld, n, diag_out);
  return cudaGetLastError();
}

#endif  // PYSA_GB_TC_E8_UNIT

template <int F, bool RND, bool E8>
static cudaError_t launch_tc_t(const TcArgs& a, int count, cudaStream_t st) {
  using C = TcCfg<F, RND, E8>;
  static bool attr_set[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !attr_set[dev]) {
    cudaError_t e = cudaFuncSetAttribute(
        k_sweep_tc<F, RND, E8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)C::BYTES);
    if (e != cudaSuccess) return e;
    attr_set[dev] = true;
  }
  k_sweep_tc<F, RND, E8><<<count, 256, C::BYTES, st>>>(a);
  return cudaGetLastError();
}

#ifdef PYSA_GB_TC_E8_UNIT
// The E4M3 variants, compiled in their own translation unit
// (sweep_tc_e8.cu) in parallel with the BF16 ones.
cudaError_t launch_tc_e8(const TcArgs& a, int F, int count, cudaStream_t st) {
  switch (F) {
    case 1: return launch_tc_t<1, false, true>(a, count, st);
    case 2: return launch_tc_t<2, false, true>(a, count, st);
    case 4: return launch_tc_t<4, false, true>(a, count, st);
  }
  return cudaErrorInvalidValue;
}
#else
cudaError_t launch_tc_e8(const TcArgs& a, int F, int count, cudaStream_t st);

cudaError_t launch_tc(const TcArgs& a, int F, bool random, int max_ctas,
                      cudaStream_t st) {
  const int64_t units = (int64_t)a.num_items * a.units_per_item;
  if (units <= 0) return cudaSuccess;
  const int count = (int)(units < max_ctas ? units : max_ctas);
  // E4M3 tiles in visiting order only (random order repacks BF16 tiles)
  if (a.e8 && !random) return launch_tc_e8(a, F, count, st);
  switch (F * 2 + (random ? 1 : 0)) {
    case 2: return launch_tc_t<1, false, false>(a, count, st);
    case 3: return launch_tc_t<1, true, false>(a, count, st);
    case 4: return launch_tc_t<2, false, false>(a, count, st);
    case 5: return launch_tc_t<2, true, false>(a, count, st);
    case 8: return launch_tc_t<4, false, false>(a, count, st);
    case 9: return launch_tc_t<4, true, false>(a, count, st);
  }
  return cudaErrorInvalidValue;
}

int tc_chains_per_cta(int n) {
  const int F = tc_fold_for(n);
  return F > 0 ? 128 / F : 0;
}
#endif  // PYSA_GB_TC_E8_UNIT

}  // namespace pysa_gb
