// Register-blocked 32-bit NTT kernels: radix-16 register sub-steps, 8 (and 16) columns per tile.
#define GSN_P32_INSTANTIATE_ET 4
#define GSN_P32_INSTANTIATE_LCG 1
#include "ntt_p32.cuh"
