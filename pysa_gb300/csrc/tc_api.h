// tc_api.h -- argument blocks of the tensor-core blocked sweep.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/pysa_gb.h"

namespace pysa_gb {

struct TcItem {
  int32_t inst, chain0, nchains, fold;
  int64_t b_off;     // element offset into the packed BF16 tiles
  int64_t diag_off;  // element offset into the packed FP32 diagonal blocks
};

struct TcArgs {
  pysa_gb_problems p;
  pysa_gb_state s;
  float* fields;
  int32_t field_ld;
  int32_t terms;  // 1: J exact in BF16; 2: J_hi + J_lo
  const uint16_t* tc_b;
  const float* tc_diag;
  const TcItem* items;
  uint64_t seed;
  int32_t recompute_every;  // >0: H and E rebuilt when sweep % this == 0
  int32_t num_items;        // items of this fold
  int32_t unit_sweeps;      // sweeps per work unit (wrap: of the launch)
  int32_t units_per_item;   // work units per item in this launch (wrap: 1)
  int32_t wrap;             // 1: wrap-around units (items of one size)
  int32_t e8;               // 1: tiles in E4M3 (visiting order only)
  int32_t fuse_exchange;    // 1: exchange inside the kernel (R | chains/CTA)
  int32_t use_pt;
  int32_t advance_counter;  // 1: the last CTA advances the sweep counter
  int32_t exchange_every;   // <= 1: every sweep; k: after (s + 1) % k == 0
  uint64_t unit_wait_ns;  // bound of the wait for an item's previous unit
                          // (0: one second)
  int32_t decision_mode;  // 0 per-block choice, 1 block rounds, 2 sub-blocks
  int32_t round_limit;    // mode 0: block rounds while the previous block's
                          // largest flip count of a chain is at most this
  int32_t* sched;  // zeroed per launch: [0] unit queue, [1] finished CTAs,
                   // [2 + item] sweeps of the item run in this launch
  // random order: permutation of (inst, sweep) at
  // perm[((sweep % perm_slots) * num_instances + inst) * max_n]; tiles and
  // diagonal blocks repacked in that order at slot sweep % rand_slots
  const int32_t* perm;
  int32_t perm_slots;
  int32_t rand_slots;
  const uint16_t* rand_b;
  const float* rand_diag;
  int64_t rand_b_stride;  // elements per slot
  int64_t rand_diag_stride;
  // optional timeline of CTA 0 (globaltimer ns): [49][24] stamps
  unsigned long long* trace;
};

// Wrap-around split of a launch's num_items * S item-sweeps over m CTAs
// (McNaughton's rule for preemptive scheduling on identical machines): share
// k holds positions [k T / m, (k + 1) T / m) of the item-major order (sweep s
// of item i at i S + s, T = num_items S), and num_items >= m makes every
// share at least S long.  Its pieces, in order: the head of the item the
// share ends in (sweeps 0 .. p1 % S - 1), its whole items, then the tail of
// the item it starts in (sweeps p0 % S .. S - 1).  That tail's head is the
// first piece of share k - 1 and, with sweeps of equal cost, is done before
// the tail starts.  Piece j of share k -> (item, first sweep, sweeps);
// false past the last piece.
__host__ __device__ inline bool wrap_piece(int items, int S, int m, int k,
                                           int j, int* it, int* sb, int* sl) {
  const int64_t T = (int64_t)items * S;
  const int64_t p0 = T * k / m, p1 = T * (k + 1) / m;
  const int head = (int)(p1 % S), tail = (int)(p0 % S);
  const int64_t f0 = (p0 + S - 1) / S, f1 = p1 / S;  // whole items [f0, f1)
  if (head) {
    if (j == 0) {
      *it = (int)(p1 / S);
      *sb = 0;
      *sl = head;
      return true;
    }
    --j;
  }
  if (j < f1 - f0) {
    *it = (int)(f0 + j);
    *sb = 0;
    *sl = S;
    return true;
  }
  if (tail && j == f1 - f0) {
    *it = (int)(p0 / S);
    *sb = tail;
    *sl = S - tail;
    return true;
  }
  return false;
}

int tc_fold_for(int n);  // 1, 2, 4 or -1 (n > 2048)
int tc_chains_per_cta(int n);
int64_t tc_b_elems(int n, int terms);
int64_t tc_diag_elems(int n);
// e8: one term in E4M3 (every coupling exact in E4M3), in the first half of
// the BF16 tiles' space.
cudaError_t launch_pack_tc(const float* Jt, int ld, int n, int terms,
                           bool e8, uint16_t* b_out, float* diag_out,
                           cudaStream_t st);
// Persistent launch over a.num_items * a.units_per_item work units with at
// most `max_ctas` CTAs (wrap: min(num_items, max_ctas) CTAs, one share of
// the item-sweeps each); a.sched must hold 2 + num_items zeroed words.
// random: visiting order from a.perm, tiles from a.rand_b / a.rand_diag.
cudaError_t launch_tc(const TcArgs& a, int F, bool random, int max_ctas,
                      cudaStream_t st);
// Tiles and diagonal blocks of every tensor-core instance (inst_off >= 0)
// in the visiting order of the current sweep and the count - 1 after it,
// into slot sweep % slots of b_out / diag_out.
cudaError_t launch_repack_tc(const pysa_gb_problems& p, int terms,
                             const int64_t* inst_off, const int32_t* perm,
                             int perm_slots, const int64_t* sweep_counter,
                             int count, int slots, uint16_t* b_out,
                             int64_t b_stride, float* diag_out,
                             int64_t diag_stride, cudaStream_t st);

}  // namespace pysa_gb
