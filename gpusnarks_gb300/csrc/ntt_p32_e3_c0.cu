// Register-blocked 32-bit NTT kernels: radix-8 register sub-steps, 4 columns per tile.
#define GSN_P32_INSTANTIATE_ET 3
#define GSN_P32_INSTANTIATE_LCG 0
#include "ntt_p32.cuh"
