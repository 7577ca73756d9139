// plain_large.cu -- plain-sweep variants for 256 < n <= 4096.
#include "plain_inst.cuh"

namespace pysa_gb {
template struct PlainLauncher<16, 8, 8, 8>;
template struct PlainLauncher<32, 4, 8, 8>;
template struct PlainLauncher<64, 2, 8, 8>;
template struct PlainLauncher<128, 1, 8, 4>;

extern const PlainVariant kPlainLarge[4] = {
    {16, 8, 8, 8, PlainLauncher<16, 8, 8, 8>::launch,
     PlainLauncher<16, 8, 8, 8>::smem, PlainLauncher<16, 8, 8, 8>::func},
    {32, 4, 8, 8, PlainLauncher<32, 4, 8, 8>::launch,
     PlainLauncher<32, 4, 8, 8>::smem, PlainLauncher<32, 4, 8, 8>::func},
    {64, 2, 8, 8, PlainLauncher<64, 2, 8, 8>::launch,
     PlainLauncher<64, 2, 8, 8>::smem, PlainLauncher<64, 2, 8, 8>::func},
    {128, 1, 8, 4, PlainLauncher<128, 1, 8, 4>::launch,
     PlainLauncher<128, 1, 8, 4>::smem, PlainLauncher<128, 1, 8, 4>::func},
};
}  // namespace pysa_gb
