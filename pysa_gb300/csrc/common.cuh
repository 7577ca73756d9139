// common.cuh -- device helpers shared by every pysa_gb300 kernel (sm_103a).
//
// * Philox4x32-10 counter-based RNG and the stream layout keyed by
//   (instance, read/chain, sweep, step), identical to the CPU oracle.
// * The Metropolis acceptance rule of pysa/ising.py:52 / pysa/qubo.py:52,
//   decided exactly as the f64 rule  log(u) < (double)beta * (double)dn
//   with an f32 fast path that only answers when its error bound allows.
// * mbarrier and bulk-copy (TMA engine, 1-D) wrappers.  Every wait is bounded:
//   on timeout the kernel records an error code in the status word and returns.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pysa_gb.h"

namespace pysa_gb {

// ------------------------------------------------------------------ Philox
__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1,
                                              uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1,
                                              uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

enum : uint32_t { TAG_SWEEP = 0, TAG_PT = 1, TAG_PERM = 2, TAG_AIS = 3,
                  TAG_PROPOSAL = 4 };

// Four consecutive draws idx = 4q..4q+3 of stream (tag, inst, a, b).
__device__ __forceinline__ void draw4(uint64_t seed, uint32_t tag,
                                      uint32_t inst, uint32_t a, uint32_t b,
                                      uint32_t q, uint32_t out[4]) {
  philox4x32_10(q, a, b, (inst << 4) | tag, (uint32_t)seed,
                (uint32_t)(seed >> 32), out);
}

// Key of chain `chain`'s sweep stream: the seed, changed by the chain's
// stream key when one is set (see pysa_gb_state.stream_key).
__device__ __forceinline__ uint64_t chain_seed(uint64_t seed,
                                               const uint32_t* key,
                                               int64_t chain) {
  if (!key) return seed;
  const uint32_t k = key[chain];
  return k ? seed ^ ((uint64_t)k * 0x9E3779B97F4A7C15ull) : seed;
}

__device__ __forceinline__ uint32_t draw1(uint64_t seed, uint32_t tag,
                                          uint32_t inst, uint32_t a,
                                          uint32_t b, uint32_t idx) {
  uint32_t o[4];
  draw4(seed, tag, inst, a, b, idx >> 2, o);
  const uint32_t k = idx & 3;
  return k == 0 ? o[0] : k == 1 ? o[1] : k == 2 ? o[2] : o[3];
}

__device__ __forceinline__ double uniform64(uint32_t x) {
  return ((double)x + 0.5) * 0x1p-32;
}

// --------------------------------------------------------------- acceptance
// Exact rule: accept iff dn >= 0 or log(u) < (double)beta * (double)dn, with
// u = (x + 0.5) 2^-32.  beta*dn is exact in f64 (24-bit x 24-bit mantissas).
// Fast path: lf = __logf(u32) has absolute error < 1e-5 over u in (0,1); the
// f32 product beta*dn has relative error < 2^-23.  Outside that band the f32
// comparison already gives the exact answer; inside it the f64 rule decides.
// The f64 rule is kept out of line: if-converted into the hot loop it would
// issue its FP64 instructions (a slow pipe on this part) on every decision.
static __device__ __noinline__ bool accept_slow(float dn, float beta, uint32_t x) {
  return log(uniform64(x)) < (double)beta * (double)dn;
}

static __device__ __noinline__ bool accept_full_slow(double full, uint32_t x) {
  return log(uniform64(x)) < full;
}

__device__ __forceinline__ bool metropolis_accept(float dn, float beta,
                                                  uint32_t x) {
  if (dn >= 0.0f) return true;
  const float bd = beta * dn;
  if (bd < -24.0f) return false;  // log(u) >= log(2^-33) > -22.9
  const float uf = __uint2float_rn(x) * 0x1p-32f + 0x1p-33f;
  const float lf = __logf(uf);
  const float margin = 3e-5f + 1e-6f * fabsf(bd);
  if (lf < bd - margin) return true;
  if (lf > bd + margin) return false;
  return accept_slow(dn, beta, x);
}

// Same rule with log(u) precomputed in f32 (lf = __logf of the f32 uniform,
// bit-identical to the value metropolis_accept forms); the rare exact f64
// decision redraws x from the stream.
static __device__ __noinline__ bool accept_slow_redraw(float dn, float beta,
                                                       uint64_t seed,
                                                       uint32_t inst,
                                                       uint32_t sweep,
                                                       uint32_t chain,
                                                       uint32_t step) {
  uint32_t o[4];
  philox4x32_10(step >> 2, sweep, chain, (inst << 4) | TAG_SWEEP,
                (uint32_t)seed, (uint32_t)(seed >> 32), o);
  const uint32_t k = step & 3;
  const uint32_t x = k == 0 ? o[0] : k == 1 ? o[1] : k == 2 ? o[2] : o[3];
  return log(uniform64(x)) < (double)beta * (double)dn;
}

__device__ __forceinline__ float log_uniform_f32(uint32_t x) {
  return __logf(__uint2float_rn(x) * 0x1p-32f + 0x1p-33f);
}

// Replica-exchange acceptance u < exp(de) (pysa/utils.py:50-55, oracle
// form), with an f32 log-domain fast path that answers only outside its
// error band.
__device__ __forceinline__ bool pt_accept_lf(float de, float lf, uint32_t x) {
  if (de >= 0.0f) return true;
  if (de < -24.0f) return false;
  const float margin = 3e-5f + 1e-6f * fabsf(de);
  if (lf < de - margin) return true;
  if (lf > de + margin) return false;
  return uniform64(x) < exp((double)de);
}
__device__ __forceinline__ bool pt_accept(float de, uint32_t x) {
  return pt_accept_lf(de, log_uniform_f32(x), x);
}

__device__ __forceinline__ bool metropolis_accept_lf(
    float dn, float beta, float lf, uint64_t seed, uint32_t inst,
    uint32_t sweep, uint32_t chain, uint32_t step) {
  if (dn >= 0.0f) return true;
  const float bd = beta * dn;
  if (bd < -24.0f) return false;
  const float margin = 3e-5f + 1e-6f * fabsf(bd);
  if (lf < bd - margin) return true;
  if (lf > bd + margin) return false;
  return accept_slow_redraw(dn, beta, seed, inst, sweep, chain, step);
}

// Same rule on a precomputed f64 threshold (AIS form: full >= 0 accepts).
__device__ __forceinline__ bool accept_full(double full, uint32_t x) {
  if (full >= 0.0) return true;
  const float ff = (float)full;
  if (ff < -24.0f) return false;
  const float uf = __uint2float_rn(x) * 0x1p-32f + 0x1p-33f;
  const float lf = __logf(uf);
  const float margin = 3e-5f + 1e-6f * fabsf(ff);
  if (lf < ff - margin) return true;
  if (lf > ff + margin) return false;
  return accept_full_slow(full, x);
}

// ------------------------------------------------------------ status word
__device__ __forceinline__ void set_status(int32_t* status, int32_t code) {
  if (status) atomicCAS(status, 0, code);
}

// ------------------------------------------------------ mbarrier / bulk copy
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx_arrive(uint64_t* bar,
                                                      uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_addr(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(
                   smem_addr(bar))
               : "memory");
}

// The waiting thread is suspended until the phase completes or about a
// millisecond passes (suspend-time hint), so waiting warps leave their
// sub-partition's issue slots to the warps that work.
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2, "
      "%3;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(1000000u)
      : "memory");
  return ok != 0;
}

// Non-blocking test of an mbarrier phase (never suspends the thread).
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar,
                                               uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.test_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait: about 2^22 polls (each try_wait already suspends for a
// hardware time slice), i.e. well over a second, then give up with a status.
constexpr uint32_t kWaitPolls = 1u << 22;

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          int32_t* status) {
  for (uint32_t i = 0; i < kWaitPolls; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  set_status(status, PYSA_GB_ERR_TIMEOUT);
  return false;
}

// 1-D bulk copy global -> shared through the TMA engine; completion is
// reported as transaction bytes on the mbarrier.  dst, src 16-B aligned and
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
                                         uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace pysa_gb
