// Register-blocked 32-bit NTT kernels: radix-16 register sub-steps, 4 columns per tile.
#define GSN_P32_INSTANTIATE_ET 4
#define GSN_P32_INSTANTIATE_LCG 0
#include "ntt_p32.cuh"
