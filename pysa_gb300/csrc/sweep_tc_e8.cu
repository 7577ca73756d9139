// sweep_tc_e8.cu -- the tensor-core sweep's E4M3-tile variants (F = 1, 2, 4,
// visiting order), compiled apart from the BF16 ones in sweep_tc.cu.
#define PYSA_GB_TC_E8_UNIT
#include "sweep_tc.cu"
