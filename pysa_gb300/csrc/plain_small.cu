// plain_small.cu -- plain-sweep variants for n <= 256.
#include "plain_inst.cuh"

namespace pysa_gb {
template struct PlainLauncher<1, 16, 4, 8>;
template struct PlainLauncher<2, 16, 4, 8>;
template struct PlainLauncher<4, 16, 4, 8>;
template struct PlainLauncher<8, 16, 4, 8>;

extern const PlainVariant kPlainSmall[4] = {
    {1, 16, 4, 8, PlainLauncher<1, 16, 4, 8>::launch,
     PlainLauncher<1, 16, 4, 8>::smem, PlainLauncher<1, 16, 4, 8>::func},
    {2, 16, 4, 8, PlainLauncher<2, 16, 4, 8>::launch,
     PlainLauncher<2, 16, 4, 8>::smem, PlainLauncher<2, 16, 4, 8>::func},
    {4, 16, 4, 8, PlainLauncher<4, 16, 4, 8>::launch,
     PlainLauncher<4, 16, 4, 8>::smem, PlainLauncher<4, 16, 4, 8>::func},
    {8, 16, 4, 8, PlainLauncher<8, 16, 4, 8>::launch,
     PlainLauncher<8, 16, 4, 8>::smem, PlainLauncher<8, 16, 4, 8>::func},
};
}  // namespace pysa_gb
