// plain_inst.cuh -- launcher template for one plain-sweep variant.
#pragma once
#include "plain_variants.h"
#include "sweep_plain.cuh"

namespace pysa_gb {

template <int NC, int GW, int W, int RB>
struct PlainLauncher {
  static size_t smem(bool random) {
    return PlainSmem<NC, GW, W, RB>::bytes(random);
  }
  static const void* func(bool random) {
    return random ? (const void*)k_sweep_plain<NC, GW, W, RB, true>
                  : (const void*)k_sweep_plain<NC, GW, W, RB, false>;
  }
  static cudaError_t launch(const PlainArgs& a, bool random, int grid,
                            cudaStream_t st) {
    const size_t sm = smem(random);
    if (random)
      k_sweep_plain<NC, GW, W, RB, true><<<grid, W * 32, sm, st>>>(a);
    else
      k_sweep_plain<NC, GW, W, RB, false><<<grid, W * 32, sm, st>>>(a);
    return cudaGetLastError();
  }
};

}  // namespace pysa_gb
